// Neighbour-list maintenance on the GPU.
//
// Reference behaviour being reproduced (wackywendell/parm):
//   NeighborList::update_list (src/trackers.cpp:19-85): a rebuild is needed
//   when the two largest displacements since the last build sum to >= skin;
//   a rebuild keeps every pair with |diff(x_i, x_j)| < (d_i + d_j)/2 + skin
//   (strict <, minimum image per OriginBox::diff, src/box.hpp:103) and not
//   excluded by NeighborList::ignore (src/trackers.hpp:190-193).
// The reference tests all N(N-1)/2 pairs.  Here a rebuild is a counting sort
// of the atoms by cell (cells no narrower than the largest list radius),
// followed by a scan of the 3^d neighbouring cells per atom.  Candidate
// distances are screened in FP32; only candidates within 2e-4 (relative) of
// the threshold are decided with the exact FP64 test, so the pair set is
// identical to the reference's.
//
// Compiled with -fmad=false: every FP64 expression here must round exactly
// like the reference's unfused CPU arithmetic.
#include "parm_check.cuh"

namespace parm {

template <int ND>
__device__ __forceinline__ typename DVec<ND>::T ldx(const void* p, uint32_t i) {
    return static_cast<const typename DVec<ND>::T*>(p)[i];
}

__device__ __forceinline__ uint32_t find_sys_of_bucket(const DevCtx& c, uint32_t b) {
    uint32_t lo = 0, hi = c.nsys;  // bucket_off[s] <= b < bucket_off[s+1]
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (c.bucket_off[mid] <= b) lo = mid; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ void posq_split(double x, float& X, float& xf) {
    double t = trunc(x * 8.0) * 0.125;   // exact: scaling by powers of two, truncation
    X = (float)t;                         // exact while |x| < 2^21
    xf = (float)(x - t);                  // x - t is exact; one rounding to FP32
}

// ---------------------------------------------------------------------------
// arm: decide, per system, whether this step starts with a rebuild
// ---------------------------------------------------------------------------
__global__ void k_arm(DevCtx c, int count_step, int use_cond, cudaGraphConditionalHandle handle) {
    __shared__ int sany;
    if (threadIdx.x == 0) sany = 0;
    __syncthreads();
    int any = 0;
    for (uint32_t s = threadIdx.x; s < c.nsys; s += blockDim.x) {
        double t1 = __longlong_as_double((long long)c.top[2 * (size_t)s]);
        double t2 = __longlong_as_double((long long)c.top[2 * (size_t)s + 1]);
        // reference: bigdist + biggestdist >= skin, evaluated only once some atom moved
        bool rb = c.force_rb[s] != 0u;
        if (!rb && t1 > 0.0) rb = __dadd_rn(__dsqrt_rn(t2), __dsqrt_rn(t1)) >= c.sys[s].skin;
        c.flag[s] = rb ? 1u : 0u;
        if (rb) {
            c.which[s] += 1u;
            c.force_rb[s] = 0u;
        }
        c.top[2 * (size_t)s] = 0ull;
        c.top[2 * (size_t)s + 1] = 0ull;
        any |= rb ? 1 : 0;
    }
    if (any) atomicOr(&sany, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        *c.any_flag = (uint32_t)sany;
        if (sany) *c.chains += 1u;
        if (count_step) c.params->step += 1ull;
        if (use_cond) cudaGraphSetConditional(handle, sany ? 1u : 0u);
    }
}

// ---------------------------------------------------------------------------
// rebuild chain (every kernel skips systems whose flag is clear)
// ---------------------------------------------------------------------------
__global__ void k_zero_cells(DevCtx c) {
    uint32_t s = blockIdx.x;
    if (!c.flag[s]) return;
    uint32_t b0 = c.bucket_off[s], nb = c.sys[s].ncell + 1;
    for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) c.cell_count[b0 + b] = 0u;
}

template <int ND>
__global__ void k_bin(DevCtx c) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    uint32_t s = c.atom_sys[i];
    if (!c.flag[s]) return;
    const SysConst& S = c.sys[s];
    uint32_t b;
    uint32_t slot;
    if (c.rank[i] == NOT_MEMBER) {
        b = c.bucket_off[s] + S.ncell;
        slot = c.nm_rank[c.orig[i]];
    } else {
        typename DVec<ND>::T xi = ldx<ND>(c.x, i);
        double xs[3] = {xi.x, xi.y, 0.0};
        if constexpr (ND == 3) xs[2] = reinterpret_cast<const double*>(&xi)[2];
        int ci[3] = {0, 0, 0};
        bool bad = false;
#pragma unroll
        for (int d = 0; d < ND; d++) {
            double t = xs[d] * S.invL[d];
            if (!isfinite(t)) { bad = true; t = 0.0; }
            double fr = t - floor(t);              // wrapped fraction in [0, 1]
            int cc = (int)(fr * (double)S.nc[d]);
            cc = cc < 0 ? 0 : (cc >= S.nc[d] ? S.nc[d] - 1 : cc);
            ci[d] = cc;
        }
        if (bad) atomicOr(c.status, ST_NONFINITE);
        b = c.bucket_off[s] + (uint32_t)((ci[2] * S.nc[1] + ci[1]) * S.nc[0] + ci[0]);
        slot = atomicAdd(&c.cell_count[b], 1u);
    }
    c.bucket[i] = b;
    c.cslot[i] = slot;
}

// exclusive scan of one system's cell counts (one CTA per system)
__global__ void __launch_bounds__(1024) k_scan_cells(DevCtx c) {
    uint32_t s = blockIdx.x;
    if (!c.flag[s]) return;
    const SysConst& S = c.sys[s];
    const uint32_t b0 = c.bucket_off[s];
    const uint32_t nb = S.ncell;  // member cells; the non-member bucket starts after them
    const uint32_t T = blockDim.x;
    const uint32_t per = (nb + T - 1) / T;
    const uint32_t lo = threadIdx.x * per;
    const uint32_t hi = min(lo + per, nb);
    uint32_t local = 0;
    for (uint32_t b = lo; b < hi; b++) local += c.cell_count[b0 + b];
    // block exclusive scan of `local`
    __shared__ uint32_t wsum[32];
    uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = local;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        uint32_t o = __shfl_up_sync(0xFFFFFFFFu, incl, off);
        if (lane >= (uint32_t)off) incl += o;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t nw = (T + 31) / 32;
        uint32_t w = lane < nw ? wsum[lane] : 0u;
        uint32_t wi = w;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            uint32_t o = __shfl_up_sync(0xFFFFFFFFu, wi, off);
            if (lane >= (uint32_t)off) wi += o;
        }
        wsum[lane] = wi - w;  // exclusive warp offsets
    }
    __syncthreads();
    uint32_t run = S.atom_off + wsum[warp] + (incl - local);
    for (uint32_t b = lo; b < hi; b++) {
        c.cell_start[b0 + b] = run;
        run += c.cell_count[b0 + b];
    }
    if (threadIdx.x == T - 1) c.cell_start[b0 + nb] = run;  // non-member bucket start
}

__global__ void k_scatter(DevCtx c) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    uint32_t s = c.atom_sys[i];
    if (!c.flag[s]) return;
    c.perm[c.cell_start[c.bucket[i]] + c.cslot[i]] = i;
}

// deterministic order inside a cell: ascending neighbour-list rank
__global__ void k_cellsort(DevCtx c) {
    uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= c.nbucket) return;
    uint32_t s = find_sys_of_bucket(c, b);
    if (!c.flag[s]) return;
    uint32_t local = b - c.bucket_off[s];
    if (local >= c.sys[s].ncell) return;  // non-member bucket is placed by nm_rank
    uint32_t lo = c.cell_start[b], hi = c.cell_start[b + 1];
    for (uint32_t k = lo + 1; k < hi; k++) {
        uint32_t v = c.perm[k];
        uint32_t key = c.rank[v];
        uint32_t m = k;
        while (m > lo) {
            uint32_t u = c.perm[m - 1];
            if (c.rank[u] <= key) break;
            c.perm[m] = u;
            m--;
        }
        c.perm[m] = v;
    }
}

template <int ND>
__global__ void k_gather(DevCtx c) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= c.n) return;
    uint32_t s = c.atom_sys[k];
    if (!c.flag[s]) return;
    using V = typename DVec<ND>::T;
    uint32_t o = c.perm[k];
    static_cast<V*>(c.x2)[k] = static_cast<const V*>(c.x)[o];
    static_cast<V*>(c.v2)[k] = static_cast<const V*>(c.v)[o];
    static_cast<V*>(c.a2)[k] = static_cast<const V*>(c.a)[o];
    static_cast<V*>(c.f2)[k] = static_cast<const V*>(c.f)[o];
    c.f32b[k] = c.f32[o];
    c.m2[k] = c.m[o];
    c.invm32b[k] = c.invm32[o];
    c.prm2[k] = c.prm[o];
    c.prm32b[k] = c.prm32[o];
    c.diam2[k] = c.diam[o];
    c.rank2[k] = c.rank[o];
    c.orig2[k] = c.orig[o];
    c.bucket2[k] = c.bucket[o];
}

template <int ND>
__global__ void k_copyback(DevCtx c) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= c.n) return;
    uint32_t s = c.atom_sys[k];
    if (!c.flag[s]) return;
    using V = typename DVec<ND>::T;
    V xk = static_cast<const V*>(c.x2)[k];
    static_cast<V*>(c.x)[k] = xk;
    static_cast<V*>(c.lastloc)[k] = xk;
    static_cast<V*>(c.v)[k] = static_cast<const V*>(c.v2)[k];
    static_cast<V*>(c.a)[k] = static_cast<const V*>(c.a2)[k];
    static_cast<V*>(c.f)[k] = static_cast<const V*>(c.f2)[k];
    c.f32[k] = c.f32b[k];
    c.m[k] = c.m2[k];
    c.invm32[k] = c.invm32b[k];
    c.prm[k] = c.prm2[k];
    c.prm32[k] = c.prm32b[k];
    double dk = c.diam2[k];
    c.diam[k] = dk;
    c.rank[k] = c.rank2[k];
    uint32_t og = c.orig2[k];
    c.orig[k] = og;
    c.slot[og] = k;
    c.bucket[k] = c.bucket2[k];
    const double* xs = reinterpret_cast<const double*>(&xk);
    float4 A, B;
    posq_split(xs[0], A.x, B.x);
    posq_split(xs[1], A.y, B.y);
    if constexpr (ND == 3) posq_split(xs[2], A.z, B.z); else { A.z = 0.f; B.z = 0.f; }
    A.w = (float)dk;
    B.w = 0.f;
    c.posA[k] = A;
    c.posB[k] = B;
}

__device__ __forceinline__ bool is_excluded(const DevCtx& c, uint32_t oi, uint32_t oj) {
    if (!c.excl_off) return false;
    for (uint32_t e = c.excl_off[oi]; e < c.excl_off[oi + 1]; e++)
        if (c.excl_list[e] == oj) return true;
    return false;
}

// full neighbour list of every member atom of a flagged system
template <int ND>
__global__ void k_build(DevCtx c) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    uint32_t s = c.atom_sys[i];
    if (!c.flag[s]) return;
    if (c.rank[i] == NOT_MEMBER) {
        c.nnb[i] = 0u;
        return;
    }
    const SysConst& S = c.sys[s];
    const uint32_t b0 = c.bucket_off[s];
    const uint32_t myb = c.bucket[i] - b0;
    int ci[3];
    ci[0] = (int)(myb % (uint32_t)S.nc[0]);
    ci[1] = (int)((myb / (uint32_t)S.nc[0]) % (uint32_t)S.nc[1]);
    ci[2] = (int)(myb / (uint32_t)(S.nc[0] * S.nc[1]));
    const float4 Ai = c.posA[i], Bi = c.posB[i];
    const double di = c.diam[i];
    const float di32 = Ai.w;
    const float skin32 = (float)S.skin;
    const uint32_t oi = c.orig[i];
    const int r0 = S.nc[0] >= 3 ? 1 : 0, r1 = S.nc[1] >= 3 ? 1 : 0;
    const int r2 = (ND == 3 && S.nc[2] >= 3) ? 1 : 0;
    uint32_t cnt = 0;
    for (int dz = -r2; dz <= r2; dz++) {
        int cz = ci[2] + dz;
        cz = cz < 0 ? cz + S.nc[2] : (cz >= S.nc[2] ? cz - S.nc[2] : cz);
        for (int dy = -r1; dy <= r1; dy++) {
            int cy = ci[1] + dy;
            cy = cy < 0 ? cy + S.nc[1] : (cy >= S.nc[1] ? cy - S.nc[1] : cy);
            for (int dx = -r0; dx <= r0; dx++) {
                int cx = ci[0] + dx;
                cx = cx < 0 ? cx + S.nc[0] : (cx >= S.nc[0] ? cx - S.nc[0] : cx);
                uint32_t cb = b0 + (uint32_t)((cz * S.nc[1] + cy) * S.nc[0] + cx);
                uint32_t js = c.cell_start[cb], je = c.cell_start[cb + 1];
                for (uint32_t j = js; j < je; j++) {
                    if (j == i) continue;
                    const float4 Aj = c.posA[j], Bj = c.posB[j];
                    float ddx = disp32(Ai.x, Aj.x, Bi.x, Bj.x, S.Lhi[0], S.Llo[0], S.invLf[0]);
                    float ddy = disp32(Ai.y, Aj.y, Bi.y, Bj.y, S.Lhi[1], S.Llo[1], S.invLf[1]);
                    float d2 = ddx * ddx + ddy * ddy;
                    if constexpr (ND == 3) {
                        float ddz = disp32(Ai.z, Aj.z, Bi.z, Bj.z, S.Lhi[2], S.Llo[2], S.invLf[2]);
                        d2 += ddz * ddz;
                    }
                    float thr = 0.5f * (di32 + Aj.w) + skin32;
                    float t2 = thr * thr;
                    bool keep;
                    if (d2 < t2 * 0.9998f) {
                        keep = true;
                    } else if (d2 > t2 * 1.0002f) {
                        keep = false;
                    } else {
                        // exact reference test: diff(x_i, x_j).norm() < (d_i + d_j)/2 + skin
                        typename DVec<ND>::T xi = ldx<ND>(c.x, i), xj = ldx<ND>(c.x, j);
                        const double* a = reinterpret_cast<const double*>(&xi);
                        const double* bb = reinterpret_cast<const double*>(&xj);
                        double r[3] = {0.0, 0.0, 0.0};
#pragma unroll
                        for (int d = 0; d < ND; d++)
                            r[d] = remainder_exact(a[d] - bb[d], S.L[d], S.invL[d], S.halfL[d]);
                        double sq = r[0] * r[0] + r[1] * r[1];
                        if constexpr (ND == 3) sq = sq + r[2] * r[2];
                        double diam = (di + c.diam[j]) / 2;
                        keep = sqrt(sq) < (diam + S.skin);
                    }
                    if (keep && is_excluded(c, oi, c.orig[j])) keep = false;
                    if (keep) {
                        if (cnt < c.maxnb) c.nbr[(size_t)cnt * c.nalloc + i] = j;
                        cnt++;
                    }
                }
            }
        }
    }
    if (cnt > c.maxnb) {
        atomicOr(c.status, ST_NBR_OVERFLOW);
        cnt = c.maxnb;
    }
    c.nnb[i] = cnt;
}

// FP64 path: order each list by neighbour-list rank, which reproduces the
// reference's summation order (pairs (i, j<i) in ascending j, then (i'>i, i)
// in ascending i').
constexpr int SORT_CAP = 256;
__global__ void k_sort_lists(DevCtx c) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    uint32_t s = c.atom_sys[i];
    if (!c.flag[s]) return;
    uint32_t cnt = c.nnb[i];
    if (cnt < 2) return;
    uint32_t key[SORT_CAP];  // lists longer than SORT_CAP are reported, not sorted
    uint32_t val[SORT_CAP];
    if (cnt > SORT_CAP) {
        atomicOr(c.status, ST_SORT_CAP);
        return;
    }
    uint32_t m = cnt;
    for (uint32_t k = 0; k < m; k++) {
        uint32_t j = c.nbr[(size_t)k * c.nalloc + i];
        uint32_t rk = c.rank[j];
        uint32_t p = k;
        while (p > 0 && key[p - 1] > rk) {
            key[p] = key[p - 1];
            val[p] = val[p - 1];
            p--;
        }
        key[p] = rk;
        val[p] = j;
    }
    for (uint32_t k = 0; k < m; k++) c.nbr[(size_t)k * c.nalloc + i] = val[k];
}

// ---------------------------------------------------------------------------
// explicit rebuild test (NeighborList::update(false) outside a time step)
// ---------------------------------------------------------------------------
template <int ND>
__global__ void k_check(DevCtx c) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool valid = false;
    double dsq = 0.0;
    uint32_t s = 0;
    if (i < c.n) {
        s = c.atom_sys[i];
        if (c.rank[i] != NOT_MEMBER) {
            dsq = disp_sq<ND>(ldx<ND>(c.x, i), ldx<ND>(c.lastloc, i));
            valid = !(dsq != dsq);
        }
    }
    check_accumulate(c, s, valid, dsq);
}

// number of half-list pairs per atom (neighbours with smaller rank)
__global__ void k_count_half(DevCtx c) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    uint32_t ri = c.rank[i];
    uint32_t cnt = 0;
    if (ri != NOT_MEMBER) {
        uint32_t nn = c.nnb[i];
        for (uint32_t k = 0; k < nn; k++)
            if (c.rank[c.nbr[(size_t)k * c.nalloc + i]] < ri) cnt++;
    }
    c.red[i] = (double)cnt;
}

template <int ND>
__global__ void k_posq(DevCtx c) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= c.n) return;
    using V = typename DVec<ND>::T;
    V xk = static_cast<const V*>(c.x)[k];
    const double* xs = reinterpret_cast<const double*>(&xk);
    float4 A, B;
    posq_split(xs[0], A.x, B.x);
    posq_split(xs[1], A.y, B.y);
    if constexpr (ND == 3) posq_split(xs[2], A.z, B.z); else { A.z = 0.f; B.z = 0.f; }
    A.w = (float)c.diam[k];
    B.w = 0.f;
    c.posA[k] = A;
    c.posB[k] = B;
}

// ---------------------------------------------------------------------------
void launch_arm(const DevCtx& c, cudaStream_t s, int count_step, int use_cond,
                unsigned long long handle) {
    k_arm<<<1, 1024, 0, s>>>(c, count_step, use_cond, (cudaGraphConditionalHandle)handle);
}

void launch_rebuild(const DevCtx& c, cudaStream_t s) {
    unsigned ga = grid_for(c.n);
    k_zero_cells<<<c.nsys, 256, 0, s>>>(c);
    if (c.nd == 3) k_bin<3><<<ga, BLOCK, 0, s>>>(c); else k_bin<2><<<ga, BLOCK, 0, s>>>(c);
    k_scan_cells<<<c.nsys, 1024, 0, s>>>(c);
    k_scatter<<<ga, BLOCK, 0, s>>>(c);
    k_cellsort<<<grid_for(c.nbucket), BLOCK, 0, s>>>(c);
    if (c.nd == 3) {
        k_gather<3><<<ga, BLOCK, 0, s>>>(c);
        k_copyback<3><<<ga, BLOCK, 0, s>>>(c);
        k_build<3><<<ga, BLOCK, 0, s>>>(c);
    } else {
        k_gather<2><<<ga, BLOCK, 0, s>>>(c);
        k_copyback<2><<<ga, BLOCK, 0, s>>>(c);
        k_build<2><<<ga, BLOCK, 0, s>>>(c);
    }
    if (c.prec == PREC_FP64) k_sort_lists<<<grid_for(c.n, 128), 128, 0, s>>>(c);
}

void launch_check(const DevCtx& c, cudaStream_t s) {
    if (c.nd == 3) k_check<3><<<grid_for(c.n), BLOCK, 0, s>>>(c);
    else k_check<2><<<grid_for(c.n), BLOCK, 0, s>>>(c);
}

void launch_numpairs(const DevCtx& c, cudaStream_t s) {
    k_count_half<<<grid_for(c.n), BLOCK, 0, s>>>(c);
}

void launch_posq(const DevCtx& c, cudaStream_t s) {
    if (c.nd == 3) k_posq<3><<<grid_for(c.n), BLOCK, 0, s>>>(c);
    else k_posq<2><<<grid_for(c.n), BLOCK, 0, s>>>(c);
}

// ---------------------------------------------------------------------------
__global__ void k_remainder_test(const double* d, const double* L, double* out, uint32_t n) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double l = L[i];
    out[i] = remainder_exact(d[i], l, 1.0 / l, 0.5 * l);
}

void launch_remainder_test(const double* d, const double* L, double* out, uint32_t n,
                           cudaStream_t s) {
    k_remainder_test<<<grid_for(n), BLOCK, 0, s>>>(d, L, out, n);
}

}  // namespace parm
