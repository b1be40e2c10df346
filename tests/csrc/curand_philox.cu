// Test-only: cuRAND's device Philox4x32-10 block function, as an independent
// implementation of the published algorithm (Salmon et al., SC'11) against
// which the library's Langevin generator is checked.  Built by the tests.
#include <cstdint>
#include <cuda_runtime.h>
#include <curand_kernel.h>

__global__ void k_curand_philox(const uint32_t* in, uint32_t* out, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t* r = in + 6 * (size_t)i;
    const uint4 c = make_uint4(r[0], r[1], r[2], r[3]);
    const uint2 k = make_uint2(r[4], r[5]);
    const uint4 o = curand_Philox4x32_10(c, k);
    out[4 * (size_t)i] = o.x;
    out[4 * (size_t)i + 1] = o.y;
    out[4 * (size_t)i + 2] = o.z;
    out[4 * (size_t)i + 3] = o.w;
}

// rows (c0, c1, c2, c3, k0, k1) in host memory -> 4 output words each; 0 on success
extern "C" int curand_philox_rows(const uint32_t* in, uint32_t* out, uint32_t n) {
    if (n == 0) return 0;
    uint32_t* buf = nullptr;
    if (cudaMalloc(&buf, 40 * (size_t)n) != cudaSuccess) return 1;
    int rc = 0;
    if (cudaMemcpy(buf, in, 24 * (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess) rc = 2;
    if (!rc) {
        k_curand_philox<<<(n + 255) / 256, 256>>>(buf, buf + 6 * (size_t)n, n);
        if (cudaGetLastError() != cudaSuccess) rc = 3;
    }
    if (!rc && cudaMemcpy(out, buf + 6 * (size_t)n, 16 * (size_t)n, cudaMemcpyDeviceToHost) != cudaSuccess) rc = 4;
    cudaFree(buf);
    return rc;
}
