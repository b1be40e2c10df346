// Kinetic energy of caller-owned device records, without any allocation.
//
// Some callers cannot allocate device memory: a host framework that owns
// every device buffer through its own pool, a real-time loop that must never
// block in the driver's allocator, or a process that runs under a fixed
// device-memory budget.  parm_kinetic_energy_noalloc serves them: it reads
// Atom records the caller already holds in device memory, writes the result
// to a device location the caller provides, and keeps its per-atom scratch
// in a file-scope __device__ array instead of allocating one.
//
// It is the same computation as parm_kinetic_energy (per-atom terms of
// AtomGroup::kinetic_energy, then one deterministic CTA reduction), on
// records in the caller's order instead of a handle's state.
#include <mutex>

#include "parm_ctx.cuh"
#include "parm_gb300.h"

namespace {

// Largest record count one call accepts: the scratch holds one double per
// atom, 2 MiB that every GPU loading this library keeps until exit.
constexpr uint32_t kNoAllocMaxAtoms = 1u << 18;

static __device__ __align__(256) double g_ke_scratch[kNoAllocMaxAtoms];

// Device address of g_ke_scratch per device (host code must not pass the
// symbol itself to a kernel: on the host it only names a stand-in object).
constexpr int kMaxDevices = 64;
std::mutex g_mutex;
double* g_scratch_ptr[kMaxDevices] = {};

__global__ void k_ke_terms(const double* atoms, uint64_t stride, uint32_t n, int nd, double o0, double o1,
                           double o2, double* scratch) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double* r = atoms + (uint64_t)i * stride;
    const double m = r[4 * nd];
    double e = 0.0;
    // AtomGroup::kinetic_energy (box.cpp:401-411): skip m == 0 or inf
    if (!(m == 0.0 || isinf(m))) {
        const double c0 = r[nd] - o0, c1 = r[nd + 1] - o1;
        double dd = __dadd_rn(__dmul_rn(c0, c0), __dmul_rn(c1, c1));
        if (nd == 3) {
            const double c2 = r[nd + 2] - o2;
            dd = __dadd_rn(dd, __dmul_rn(c2, c2));
        }
        e = __dmul_rn(m / 2, dd);
    }
    scratch[i] = e;
}

__global__ void __launch_bounds__(1024) k_ke_reduce(const double* scratch, uint32_t n, double* out) {
    __shared__ double sh[32];
    double acc = 0.0;
    for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) acc += scratch[k];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xFFFFFFFFu, acc, off);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, off);
        if (threadIdx.x == 0) *out = v;
    }
}

int scratch_for_current_device(double** p) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return parm::set_error(PARM_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return parm::set_error(PARM_ERR_RUNTIME, "device index out of range");
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_ptr[dev]) {
        void* q = nullptr;
        e = cudaGetSymbolAddress(&q, g_ke_scratch);
        if (e != cudaSuccess) return parm::set_error(PARM_ERR_CUDA, cudaGetErrorString(e));
        g_scratch_ptr[dev] = static_cast<double*>(q);
    }
    *p = g_scratch_ptr[dev];
    return PARM_OK;
}

}  // namespace

extern "C" int parm_kinetic_energy_noalloc(const double* atoms, uint64_t stride, uint32_t natoms, int ndim,
                                           const double* origin, double* out, void* stream) {
    if (!atoms || !out) return parm::set_error(PARM_ERR_ARG, "NULL argument");
    if (ndim != 2 && ndim != 3) return parm::set_error(PARM_ERR_ARG, "ndim must be 2 or 3");
    if (stride < 4 * (uint64_t)ndim + 1) return parm::set_error(PARM_ERR_ARG, "stride smaller than an Atom record");
    if (natoms > kNoAllocMaxAtoms)
        return parm::set_error(PARM_ERR_ARG, "parm_kinetic_energy_noalloc: at most 262144 atoms per call "
                                             "(the size of its static scratch)");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (s) {
        // the scratch address belongs to the current device; a stream of another device cannot use it
        int sdev = -1, cur = -1;
        cudaError_t e = cudaStreamGetDevice(s, &sdev);
        if (e != cudaSuccess) return parm::set_error(PARM_ERR_ARG, cudaGetErrorString(e));
        e = cudaGetDevice(&cur);
        if (e != cudaSuccess) return parm::set_error(PARM_ERR_CUDA, cudaGetErrorString(e));
        if (sdev != cur)
            return parm::set_error(PARM_ERR_ARG, "parm_kinetic_energy_noalloc: the stream belongs to another "
                                                 "device than the current one");
    }
    double* scratch = nullptr;
    int r = scratch_for_current_device(&scratch);
    if (r != PARM_OK) return r;
    const double o0 = origin ? origin[0] : 0.0, o1 = origin ? origin[1] : 0.0;
    const double o2 = (origin && ndim == 3) ? origin[2] : 0.0;
    if (natoms) k_ke_terms<<<parm::grid_for(natoms), parm::BLOCK, 0, s>>>(atoms, stride, natoms, ndim, o0, o1, o2, scratch);
    k_ke_reduce<<<1, 1024, 0, s>>>(scratch, natoms, out);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return parm::set_error(PARM_ERR_CUDA, cudaGetErrorString(e));
    return PARM_OK;
}
