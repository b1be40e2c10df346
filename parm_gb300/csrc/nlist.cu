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
        if (count_step && !c.active[s]) {
            // frozen system: no rebuild in time steps; its pending test
            // (displacements, forced rebuild) waits until it is stepped again
            c.flag[s] = 0u;
            continue;
        }
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
    // every lane of the warp reaches the cell-count update below (the grid is
    // whole warps), so the lanes that bin a member can be counted by a ballot
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t s = i < c.n ? c.atom_sys[i] : 0u;
    const bool live = i < c.n && c.flag[s];
    const bool member = live && c.rank[i] != NOT_MEMBER;
    uint32_t b = 0u, slot = 0u;
    if (live && !member) {
        b = c.bucket_off[s] + c.sys[s].ncell;
        slot = c.nm_rank[c.orig[i]];
    }
    if (member) {
        const SysConst& S = c.sys[s];
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
    }
    // one atomic per distinct cell of the warp (atoms arrive in cell order,
    // so a warp holds two or three cells): the lanes of a cell take
    // consecutive slots from its count
    const uint32_t mem = __ballot_sync(0xFFFFFFFFu, member);
    if (member) {
        const uint32_t lane = threadIdx.x & 31u;
        const uint32_t peers = __match_any_sync(mem, b);
        const uint32_t leader = (uint32_t)__ffs(peers) - 1u;
        uint32_t first = 0u;
        if (lane == leader) first = atomicAdd(&c.cell_count[b], (uint32_t)__popc(peers));
        first = __shfl_sync(peers, first, leader);
        slot = first + (uint32_t)__popc(peers & ((1u << lane) - 1u));
    }
    if (live) {
        c.bucket[i] = b;
        c.cslot[i] = slot;
    }
}

// ---------------------------------------------------------------------------
// Cell offsets: a segmented exclusive scan of the bucket counts over all
// buckets, one segment per system (its first bucket starts a segment), in
// three passes (block aggregates, scan of aggregates, final offsets).  Only
// buckets of flagged systems are written; other systems' counts are stale but
// never cross a segment boundary.
// ---------------------------------------------------------------------------
constexpr int SCAN_THREADS = 512;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_CHUNK = SCAN_THREADS * SCAN_ITEMS;

struct SegPair {
    uint32_t f;  // segment starts in this span
    uint32_t v;  // sum since the last segment start
};

__device__ __forceinline__ SegPair seg_combine(SegPair a, SegPair b) {
    return {a.f | b.f, b.f ? b.v : a.v + b.v};
}

// block-wide inclusive scan of one pair per thread; returns the exclusive
// carry for this thread and the block aggregate
__device__ __forceinline__ SegPair seg_block_scan(SegPair x, SegPair& aggregate) {
    __shared__ SegPair wsum[SCAN_THREADS / 32];
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    SegPair inc = x;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        SegPair o;
        o.f = __shfl_up_sync(0xFFFFFFFFu, inc.f, off);
        o.v = __shfl_up_sync(0xFFFFFFFFu, inc.v, off);
        if (lane >= (unsigned)off) inc = seg_combine(o, inc);
    }
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        SegPair w = lane < SCAN_THREADS / 32 ? wsum[lane] : SegPair{0u, 0u};
        SegPair wi = w;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            SegPair o;
            o.f = __shfl_up_sync(0xFFFFFFFFu, wi.f, off);
            o.v = __shfl_up_sync(0xFFFFFFFFu, wi.v, off);
            if (lane >= (unsigned)off) wi = seg_combine(o, wi);
        }
        if (lane < SCAN_THREADS / 32) wsum[lane] = wi;   // inclusive over warps
    }
    __syncthreads();
    aggregate = wsum[SCAN_THREADS / 32 - 1];
    // exclusive carry = (inclusive of previous warps) + (inclusive of earlier lanes)
    SegPair prev_w = warp > 0 ? wsum[warp - 1] : SegPair{0u, 0u};
    SegPair prev_l;
    prev_l.f = __shfl_up_sync(0xFFFFFFFFu, inc.f, 1);
    prev_l.v = __shfl_up_sync(0xFFFFFFFFu, inc.v, 1);
    if (lane == 0) prev_l = SegPair{0u, 0u};
    SegPair carry = seg_combine(prev_w, prev_l);
    __syncthreads();
    return carry;
}

__device__ __forceinline__ SegPair bucket_item(const DevCtx& c, uint32_t b) {
    if (b >= c.nbucket) return {0u, 0u};
    const uint32_t s = c.bucket_sys[b];
    return {b == c.bucket_off[s] ? 1u : 0u, c.cell_count[b]};
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_blocks(DevCtx c) {
    const uint32_t base = blockIdx.x * SCAN_CHUNK + threadIdx.x * SCAN_ITEMS;
    SegPair t{0u, 0u};
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) t = seg_combine(t, bucket_item(c, base + k));
    SegPair agg;
    seg_block_scan(t, agg);
    if (threadIdx.x == 0) {
        c.scan_aux[2 * blockIdx.x] = agg.f;
        c.scan_aux[2 * blockIdx.x + 1] = agg.v;
    }
}

// exclusive segmented scan of the block aggregates (one CTA)
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_aux(DevCtx c, uint32_t nblk) {
    SegPair run{0u, 0u};
    for (uint32_t b0 = 0; b0 < nblk; b0 += SCAN_THREADS) {
        const uint32_t b = b0 + threadIdx.x;
        SegPair x = b < nblk ? SegPair{c.scan_aux[2 * b], c.scan_aux[2 * b + 1]} : SegPair{0u, 0u};
        SegPair agg;
        SegPair carry = seg_block_scan(x, agg);
        SegPair excl = seg_combine(run, carry);
        if (b < nblk) {
            c.scan_aux[2 * b] = excl.f;
            c.scan_aux[2 * b + 1] = excl.v;
        }
        run = seg_combine(run, agg);
    }
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_write(DevCtx c) {
    const uint32_t base = blockIdx.x * SCAN_CHUNK + threadIdx.x * SCAN_ITEMS;
    SegPair items[SCAN_ITEMS];
    SegPair t{0u, 0u};
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        items[k] = bucket_item(c, base + k);
        t = seg_combine(t, items[k]);
    }
    SegPair agg;
    SegPair carry = seg_block_scan(t, agg);
    SegPair run = seg_combine(SegPair{c.scan_aux[2 * blockIdx.x], c.scan_aux[2 * blockIdx.x + 1]}, carry);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        const uint32_t b = base + k;
        if (b >= c.nbucket) break;
        const uint32_t excl = items[k].f ? 0u : run.v;   // exclusive, restarted per system
        run = seg_combine(run, items[k]);
        const uint32_t s = c.bucket_sys[b];
        if (c.flag[s]) c.cell_start[b] = c.sys[s].atom_off + excl;
    }
}

__global__ void k_scatter(DevCtx c) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    uint32_t s = c.atom_sys[i];
    if (!c.flag[s]) return;
    c.perm[c.cell_start[c.bucket[i]] + c.cslot[i]] = i;
}

// deterministic order inside a cell: ascending neighbour-list rank.  One warp
// per cell: each lane holds one atom of the cell and counts the atoms ranked
// before it (cells of up to 32 atoms; larger cells are sorted by lane 0).
__global__ void k_cellsort(DevCtx c) {
    const uint32_t b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (b >= c.nbucket) return;   // uniform in the warp
    const uint32_t s = find_sys_of_bucket(c, b);
    if (!c.flag[s]) return;
    const uint32_t local = b - c.bucket_off[s];
    if (local >= c.sys[s].ncell) return;  // non-member bucket is placed by nm_rank
    const uint32_t lo = c.cell_start[b], hi = c.cell_start[b + 1];
    const uint32_t cnt = hi - lo;
    if (cnt < 2) return;
    if (cnt <= 32u) {
        const uint32_t v = lane < cnt ? c.perm[lo + lane] : 0u;
        const uint32_t rk = lane < cnt ? c.rank[v] : 0xFFFFFFFFu;
        uint32_t pos = 0;
        for (uint32_t j = 0; j < cnt; j++) {
            const uint32_t kj = __shfl_sync(0xFFFFFFFFu, rk, j);
            pos += (kj < rk || (kj == rk && j < lane)) ? 1u : 0u;
        }
        __syncwarp();
        if (lane < cnt) c.perm[lo + pos] = v;
        return;
    }
    if (lane != 0) return;
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
    if (c.prec != PREC_MIXED) static_cast<V*>(c.f2)[k] = static_cast<const V*>(c.f)[o];   // FP64 forces: FP64 path only
    c.f32b[k] = c.f32[o];
    // arrays whose entries are all equal are left as they are (copy back too)
    if (*c.m_mixed) {
        c.m2[k] = c.m[o];
        c.invm32b[k] = c.invm32[o];
    }
    if (!c.same_prm) {
        c.prm2[k] = c.prm[o];
        c.prm32b[k] = c.prm32[o];
        c.diam2[k] = c.diam[o];
    }
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
    if (c.prec != PREC_MIXED) static_cast<V*>(c.f)[k] = static_cast<const V*>(c.f2)[k];
    c.f32[k] = c.f32b[k];
    if (*c.m_mixed) {
        c.m[k] = c.m2[k];
        c.invm32[k] = c.invm32b[k];
    }
    double dk;
    if (!c.same_prm) {
        c.prm[k] = c.prm2[k];
        c.prm32[k] = c.prm32b[k];
        dk = c.diam2[k];
        c.diam[k] = dk;
    } else {
        dk = c.diam[k];   // every atom's
    }
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
    c.pos[2 * (size_t)(k)] = A;
    c.pos[2 * (size_t)(k) + 1] = B;
    if (c.staged) {
        // cell-block record in the frame of this build
        float4 fr = make_float4(0.f, 0.f, 0.f, __uint_as_float(REC_BIAS | (REC_BIAS << 12) | (REC_BIAS << 22)));
        if (c.rank[k] != NOT_MEMBER) {
            const SysConst& S = c.sys[s];
            uint32_t ci[3];
            cell_coords(S, c.bucket[k] - c.bucket_off[s], ci);
            bool ok;
            fr = rec_frame<ND>(S, ci, A, B, ok);
            if (!ok) atomicOr(c.status, ST_IMAGE_RANGE);
        }
        c.rframe[k] = fr;
        c.rec[k] = make_record(A, B, fr);
    }
    // position relative to the lower corner of its cell, for the warp list
    // build (the cell-block build stages its own positions)
    if (!c.staged && c.rank[k] != NOT_MEMBER) {
        const SysConst& S = c.sys[s];
        const uint32_t myb = c.bucket[k] - c.bucket_off[s];
        const uint32_t ci[3] = {myb % (uint32_t)S.nc[0], (myb / (uint32_t)S.nc[0]) % (uint32_t)S.nc[1],
                                myb / (uint32_t)(S.nc[0] * S.nc[1])};
        float pr[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int d = 0; d < ND; d++) {
            double t = xs[d] * S.invL[d];
            double fr = t - floor(t);
            pr[d] = (float)(fr * S.L[d] - (double)ci[d] * S.cellw[d]);
        }
        c.posw[k] = make_float4(pr[0], pr[1], pr[2], (float)dk);
    }
}

__device__ __forceinline__ bool is_excluded(const DevCtx& c, uint32_t oi, uint32_t oj) {
    if (!c.excl_off) return false;
    for (uint32_t e = c.excl_off[oi]; e < c.excl_off[oi + 1]; e++)
        if (c.excl_list[e] == oj) return true;
    return false;
}

// exact reference test: diff(x_i, x_j).norm() < (d_i + d_j)/2 + skin
template <int ND>
__device__ __noinline__ bool keep_exact(const DevCtx& c, const SysConst& S, uint32_t i, uint32_t j) {
    typename DVec<ND>::T xi = ldx<ND>(c.x, i), xj = ldx<ND>(c.x, j);
    const double* a = reinterpret_cast<const double*>(&xi);
    const double* bb = reinterpret_cast<const double*>(&xj);
    double r[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int d = 0; d < ND; d++) r[d] = remainder_exact(a[d] - bb[d], S.L[d], S.invL[d], S.halfL[d]);
    double sq = r[0] * r[0] + r[1] * r[1];
    if constexpr (ND == 3) sq = sq + r[2] * r[2];
    double diam = (c.diam[i] + c.diam[j]) / 2;
    return sqrt(sq) < (diam + S.skin);
}

// Full neighbour lists of a flagged system's member atoms (row-major:
// nbr[i * maxnb + k]), one warp per cell with warp-ballot compaction.
// The candidates of the 3^d stencil cells are numbered consecutively (stencil
// order, then cell order); the warp takes 32 candidates at a time, one per
// lane, and tests all of them against each home atom in turn.  The accepted
// candidates of a home atom are appended in candidate order by a ballot and a
// population count, so the lists are deterministic and written coalesced.
// Positions are relative to each cell's lower corner: a candidate in the
// stencil cell at offset (dx,dy,dz) is displaced by (dx,dy,dz) * cell width in
// the periodic continuation of the grid (axes with a single cell take a
// per-pair minimum image instead).  Distances are screened in FP32; candidates
// within 2e-4 (relative) of the threshold get the exact FP64 reference test.
constexpr int BUILD_WARPS = 4;
template <int ND, bool WRAP>
__global__ void __launch_bounds__(BUILD_WARPS * 32) k_build(DevCtx c) {
    __shared__ float4 home[BUILD_WARPS][32];
    __shared__ uint32_t pre[BUILD_WARPS][32];
    __shared__ uint32_t jst[BUILD_WARPS][32];
    __shared__ float4 soff[BUILD_WARPS][32];
    const uint32_t lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
    const uint32_t b = blockIdx.x * BUILD_WARPS + wib;   // one warp per bucket
    if (b >= c.nbucket) return;
    const uint32_t s = c.bucket_sys[b];
    if (!c.flag[s]) return;
    const SysConst& S = c.sys[s];
    const uint32_t b0 = c.bucket_off[s];
    const uint32_t myb = b - b0;
    if (myb >= S.ncell) {
        // non-member bucket: these atoms have no neighbours
        for (uint32_t i = c.cell_start[b] + lane; i < S.atom_off + S.natoms; i += 32) c.nnb[i] = 0u;
        return;
    }
    const uint32_t cs = c.cell_start[b], ce = c.cell_start[b + 1];
    if (cs == ce) return;
    const int nc0 = S.nc[0], nc1 = S.nc[1], nc2 = S.nc[2];
    const int ci0 = (int)(myb % (uint32_t)nc0);
    const int ci1 = (int)((myb / (uint32_t)nc0) % (uint32_t)nc1);
    const int ci2 = (int)(myb / (uint32_t)(nc0 * nc1));
    const int r0 = nc0 >= 3 ? 1 : 0, r1 = nc1 >= 3 ? 1 : 0;
    const int r2 = (ND == 3 && nc2 >= 3) ? 1 : 0;
    const int w0 = 2 * r0 + 1, w1 = 2 * r1 + 1, w2 = 2 * r2 + 1;
    const uint32_t nst = (uint32_t)(w0 * w1 * w2);
    // stencil table: lane t describes stencil cell t
    uint32_t cntl = 0;
    if (lane < nst) {
        const int dx = (int)(lane % (uint32_t)w0) - r0;
        const int dy = (int)((lane / (uint32_t)w0) % (uint32_t)w1) - r1;
        const int dz = (int)(lane / (uint32_t)(w0 * w1)) - r2;
        int cx = ci0 + dx, cy = ci1 + dy, cz = ci2 + dz;
        cx = cx < 0 ? cx + nc0 : (cx >= nc0 ? cx - nc0 : cx);
        cy = cy < 0 ? cy + nc1 : (cy >= nc1 ? cy - nc1 : cy);
        cz = cz < 0 ? cz + nc2 : (cz >= nc2 ? cz - nc2 : cz);
        const uint32_t cb = b0 + (uint32_t)((cz * nc1 + cy) * nc0 + cx);
        const uint32_t js = c.cell_start[cb];
        cntl = c.cell_start[cb + 1] - js;
        jst[wib][lane] = js;
        soff[wib][lane] = make_float4((float)dx * S.cellw32[0], (float)dy * S.cellw32[1],
                                      (float)dz * S.cellw32[2], 0.f);
    }
    uint32_t incl = cntl;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (uint32_t)o) incl += t;
    }
    pre[wib][lane] = incl - cntl;
    const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    __syncwarp();

    // per-pair minimum image only along axes with a single cell (WRAP kernels)
    const bool wrap0 = WRAP && r0 == 0, wrap1 = WRAP && r1 == 0, wrap2 = WRAP && (ND == 3) && r2 == 0;
    const float kShift = 12582912.0f;
    const float skin32 = (float)S.skin;
    const bool uni_thr = c.uniform & UNI_DIAM;
    const uint32_t maxnb = c.maxnb;
    for (uint32_t hb = cs; hb < ce; hb += 32) {
        const uint32_t mh = min(32u, ce - hb);
        if (lane < mh) home[wib][lane] = c.posw[hb + lane];
        uint32_t mycnt = 0;   // neighbours found so far for home atom hb + lane
        __syncwarp();
        const float4 H0 = home[wib][0];
        const float t2u = (H0.w + skin32) * (H0.w + skin32);
        for (uint32_t base = 0; base < total; base += 32) {
            const uint32_t q = base + lane;
            const bool valid = q < total;
            uint32_t j = 0xFFFFFFFFu;
            float4 Q = make_float4(0.f, 0.f, 0.f, 0.f);
            if (valid) {
                uint32_t st = 0;
#pragma unroll 1
                for (uint32_t k = 1; k < nst; k++)
                    if (pre[wib][k] <= q) st = k;
                j = jst[wib][st] + (q - pre[wib][st]);
                const float4 R = c.posw[j];
                const float4 O = soff[wib][st];
                Q = make_float4(R.x + O.x, R.y + O.y, R.z + O.z, R.w);
            }
            for (uint32_t h = 0; h < mh; h++) {
                const float4 P = home[wib][h];
                float d0 = P.x - Q.x, d1 = P.y - Q.y, d2c = 0.f;
                if (wrap0) d0 = __fmaf_rn(-__fsub_rn(__fmaf_rn(d0, S.invLf[0], kShift), kShift), S.Lhi[0], d0);
                if (wrap1) d1 = __fmaf_rn(-__fsub_rn(__fmaf_rn(d1, S.invLf[1], kShift), kShift), S.Lhi[1], d1);
                if constexpr (ND == 3) {
                    d2c = P.z - Q.z;
                    if (wrap2) d2c = __fmaf_rn(-__fsub_rn(__fmaf_rn(d2c, S.invLf[2], kShift), kShift), S.Lhi[2], d2c);
                }
                const float rr = d0 * d0 + d1 * d1 + d2c * d2c;
                float t2 = t2u;
                if (!uni_thr) {
                    const float thr = 0.5f * (P.w + Q.w) + skin32;
                    t2 = thr * thr;
                }
                const uint32_t i = hb + h;
                bool keep = valid && rr < t2 * 0.9998f && j != i;
                const bool band = valid && !keep && rr <= t2 * 1.0002f && j != i;
                if (__any_sync(0xFFFFFFFFu, band)) {   // rare: exact reference test
                    if (band) keep = keep_exact<ND>(c, S, i, j);
                }
                if (c.excl_off) {
                    if (keep && is_excluded(c, c.orig[i], c.orig[j])) keep = false;
                }
                const uint32_t mask = __ballot_sync(0xFFFFFFFFu, keep);
                if (mask) {
                    const uint32_t ch = __shfl_sync(0xFFFFFFFFu, mycnt, h);
                    if (keep) {
                        const uint32_t pos = ch + __popc(mask & ((1u << lane) - 1u));
                        if (pos < maxnb) c.nbr[(size_t)i * maxnb + pos] = j;
                    }
                    if (lane == h) mycnt += __popc(mask);
                }
            }
        }
        if (lane < mh) {
            if (mycnt > maxnb) {
                atomicOr(c.status, ST_NBR_OVERFLOW);
                mycnt = maxnb;
            }
            c.nnb[hb + lane] = mycnt;
        }
        __syncwarp();
    }
}

// All-pairs list build of the handles with a LeesEdwardsBox (FP64 path): the
// sheared images do not follow the cell stencil, so every member atom tests
// every member of its system with the reference's own test (trackers.cpp:
// 59-69: diff(x_i, x_j).norm() < (d_i + d_j)/2 + skin), as the reference's
// O(N^2) list build does; k_sort_lists then orders each list by rank.
template <int ND>
__global__ void k_build_lees(DevCtx c) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const uint32_t s = c.atom_sys[i];
    if (!c.flag[s]) return;
    if (c.rank[i] == NOT_MEMBER) {
        c.nnb[i] = 0u;
        return;
    }
    const SysConst& S = c.sys[s];
    typename DVec<ND>::T xv = ldx<ND>(c.x, i);
    const double* xi = reinterpret_cast<const double*>(&xv);
    const double di = c.diam[i];
    const uint32_t maxnb = c.maxnb;
    uint32_t cnt = 0;
    for (uint32_t j = S.atom_off; j < S.atom_off + S.natoms; j++) {
        if (j == i || c.rank[j] == NOT_MEMBER) continue;
        typename DVec<ND>::T yv = ldx<ND>(c.x, j);
        const double* xj = reinterpret_cast<const double*>(&yv);
        double r[3] = {0.0, 0.0, 0.0};
        if (S.lees) {
            lees_diff<ND>(S, xi, xj, r);
        } else {
#pragma unroll
            for (int d = 0; d < ND; d++) r[d] = remainder_exact(xi[d] - xj[d], S.L[d], S.invL[d], S.halfL[d]);
        }
        double sq = r[0] * r[0] + r[1] * r[1];
        if constexpr (ND == 3) sq = sq + r[2] * r[2];
        const double diam = (di + c.diam[j]) / 2;
        if (!(sqrt(sq) < (diam + S.skin))) continue;
        if (c.excl_off && is_excluded(c, c.orig[i], c.orig[j])) continue;
        if (cnt < maxnb) c.nbr[(size_t)i * maxnb + cnt] = j;
        cnt++;
    }
    if (cnt > maxnb) {
        atomicOr(c.status, ST_NBR_OVERFLOW);
        cnt = maxnb;
    }
    c.nnb[i] = cnt;
}

// ---------------------------------------------------------------------------
// Shared-memory tiles for the mixed-precision pair kernel (built after the
// lists).  A tile is TILE_ATOMS consecutive atoms of one system.  Its frame
// origin is the coarse position A0 of its first atom; atom i sits in the frame
// at X_i - m_i L (m_i rounds (X_i - A0)/L), and its neighbour j, whose pair
// image is n_ij = round((X_i - X_j)/L), at X_j + (n_ij - m_i) L.  The tile's
// entries are its distinct (j, n_ij - m_i) pairs (deduplicated through a
// shared-memory hash table) and the tile lists hold 16-bit entry numbers.
// Images are stored as 8-bit signed numbers per axis.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t img_code(int a, int b, int c) {
    return (uint32_t)(a + 128) | ((uint32_t)(b + 128) << 8) | ((uint32_t)(c + 128) << 16);
}

__device__ __forceinline__ float round_ratio(float num, float inv) {
    const float kShift = 12582912.0f;
    return __fsub_rn(__fmaf_rn(num, inv, kShift), kShift);
}

__device__ __forceinline__ uint32_t hash_slot(unsigned long long key) {
    return (uint32_t)((key * 0x9E3779B97F4A7C15ull) >> 52) & (TILE_HASH - 1);
}

constexpr unsigned long long HASH_EMPTY = ~0ull;

template <int ND>
__global__ void __launch_bounds__(TILE_ATOMS) k_tile(DevCtx c, int all) {
    __shared__ unsigned long long hkey[TILE_HASH];
    __shared__ uint16_t hidx[TILE_HASH];
    __shared__ uint32_t wsum[TILE_ATOMS / 32];
    const uint32_t t = blockIdx.x;
    if (t >= c.ntile) return;
    const uint32_t s = c.tile_sys[t];
    if (!all && !c.flag[s]) return;
    const SysConst& S = c.sys[s];
    const uint32_t a0 = c.tile_atom0[t], na = c.tile_natom[t];
    const uint32_t tid = threadIdx.x;
    for (uint32_t q = tid; q < TILE_HASH; q += blockDim.x) hkey[q] = HASH_EMPTY;
    const float4 A0 = c.pos[2 * (size_t)a0];
    __syncthreads();
    const uint32_t i = a0 + tid;
    const bool act = tid < na && c.rank[i] != NOT_MEMBER;
    int m[3] = {0, 0, 0};
    uint32_t nn = 0;
    bool bad = false;
    float4 Ai = make_float4(0.f, 0.f, 0.f, 0.f);
    if (act) {
        Ai = c.pos[2 * (size_t)i];
        m[0] = (int)round_ratio(Ai.x - A0.x, S.invLf[0]);
        m[1] = (int)round_ratio(Ai.y - A0.y, S.invLf[1]);
        if (ND == 3) m[2] = (int)round_ratio(Ai.z - A0.z, S.invLf[2]);
        nn = c.nnb[i];
        for (uint32_t k = 0; k < nn; k++) {
            const uint32_t j = c.nbr[(size_t)i * c.maxnb + k];
            const float4 Aj = c.pos[2 * (size_t)j];
            int im[3] = {0, 0, 0};
            im[0] = (int)round_ratio(Ai.x - Aj.x, S.invLf[0]) - m[0];
            im[1] = (int)round_ratio(Ai.y - Aj.y, S.invLf[1]) - m[1];
            if (ND == 3) im[2] = (int)round_ratio(Ai.z - Aj.z, S.invLf[2]) - m[2];
            if (im[0] < -127 || im[0] > 127 || im[1] < -127 || im[1] > 127 || im[2] < -127 || im[2] > 127)
                bad = true;
            const unsigned long long key = ((unsigned long long)j << 24) | img_code(im[0], im[1], im[2]);
            uint32_t slot = hash_slot(key);
            bool placed = false;
            for (uint32_t p = 0; p < TILE_HASH; p++) {   // bounded linear probing
                const unsigned long long old = atomicCAS(&hkey[slot], HASH_EMPTY, key);
                if (old == HASH_EMPTY || old == key) {
                    placed = true;
                    break;
                }
                slot = (slot + 1) & (TILE_HASH - 1);
            }
            if (!placed) bad = true;
        }
        if (m[0] < -127 || m[0] > 127 || m[1] < -127 || m[1] > 127 || m[2] < -127 || m[2] > 127) bad = true;
        c.atom_img[i] = img_code(m[0], m[1], m[2]);
    }
    if (bad) atomicOr(c.status, ST_IMAGE_RANGE | ST_TILE_OVERFLOW);
    __syncthreads();
    // compact the occupied slots into entry numbers (block exclusive scan)
    constexpr uint32_t PER = TILE_HASH / TILE_ATOMS;
    uint32_t cnt = 0;
    for (uint32_t q = 0; q < PER; q++) cnt += hkey[tid * PER + q] != HASH_EMPTY;
    const uint32_t lane = tid & 31u, warp = tid >> 5;
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (uint32_t)o) incl += v;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    uint32_t base = incl - cnt;
    for (uint32_t w = 0; w < warp; w++) base += wsum[w];
    uint32_t total = 0;
    for (uint32_t w = 0; w < TILE_ATOMS / 32; w++) total += wsum[w];
    for (uint32_t q = 0; q < PER; q++) {
        const uint32_t slot = tid * PER + q;
        const unsigned long long key = hkey[slot];
        if (key == HASH_EMPTY) continue;
        if (base < TILE_ECAP) c.tile_ent[(size_t)t * TILE_ECAP + base] = key;
        hidx[slot] = (uint16_t)min(base, (uint32_t)TILE_ECAP - 1u);
        base++;
    }
    if (tid == 0) {
        c.tile_ne[t] = min(total, (uint32_t)TILE_ECAP);
        c.tile_anchor[t] = A0;
        if (total > TILE_ECAP) atomicOr(c.status, ST_TILE_OVERFLOW);
    }
    __syncthreads();
    // tile lists: entry number of every (atom, neighbour)
    if (act) {
        uint16_t* lst = c.tile_lst + (size_t)t * c.maxnb * TILE_ATOMS + tid;
        for (uint32_t k = 0; k < nn; k++) {
            const uint32_t j = c.nbr[(size_t)i * c.maxnb + k];
            const float4 Aj = c.pos[2 * (size_t)j];
            int im[3] = {0, 0, 0};
            im[0] = (int)round_ratio(Ai.x - Aj.x, S.invLf[0]) - m[0];
            im[1] = (int)round_ratio(Ai.y - Aj.y, S.invLf[1]) - m[1];
            if (ND == 3) im[2] = (int)round_ratio(Ai.z - Aj.z, S.invLf[2]) - m[2];
            const unsigned long long key = ((unsigned long long)j << 24) | img_code(im[0], im[1], im[2]);
            uint32_t slot = hash_slot(key);
            uint16_t e = 0;
            for (uint32_t p = 0; p < TILE_HASH; p++) {
                const unsigned long long kk = hkey[slot];
                if (kk == key) {
                    e = hidx[slot];
                    break;
                }
                if (kk == HASH_EMPTY) break;
                slot = (slot + 1) & (TILE_HASH - 1);
            }
            lst[(size_t)k * TILE_ATOMS] = e;
        }
    }
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
        uint32_t j = c.nbr[(size_t)i * c.maxnb + k];
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
    for (uint32_t k = 0; k < m; k++) c.nbr[(size_t)i * c.maxnb + k] = val[k];
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
            if (c.rank[c.nbr[(size_t)i * c.maxnb + k]] < ri) cnt++;
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
    c.pos[2 * (size_t)(k)] = A;
    c.pos[2 * (size_t)(k) + 1] = B;
    if (c.staged) c.rec[k] = make_record(A, B, c.rframe[k]);
}

// the cell-block records of every atom in the frames of the current cells
// (after a box change on the same cell grids, or when the mixed path moves to
// the cell-block kernels between list builds)
template <int ND>
__global__ void k_reframe(DevCtx c) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= c.n) return;
    const uint32_t s = c.atom_sys[k];
    float4 A, B;
    ld_pos(c.pos, k, A, B);
    float4 fr = make_float4(0.f, 0.f, 0.f, __uint_as_float(REC_BIAS | (REC_BIAS << 12) | (REC_BIAS << 22)));
    if (c.rank[k] != NOT_MEMBER) {
        const SysConst& S = c.sys[s];
        uint32_t ci[3];
        cell_coords(S, c.bucket[k] - c.bucket_off[s], ci);
        bool ok;
        fr = rec_frame<ND>(S, ci, A, B, ok);
    }
    c.rframe[k] = fr;
    c.rec[k] = make_record(A, B, fr);
}

// ---------------------------------------------------------------------------
void launch_tiles(const DevCtx& c, cudaStream_t s, int all);

void launch_arm(const DevCtx& c, cudaStream_t s, int count_step, int use_cond,
                unsigned long long handle) {
    const unsigned threads = c.nsys <= 32 ? 32u : (c.nsys <= 256 ? 256u : 1024u);
    k_arm<<<1, threads, 0, s>>>(c, count_step, use_cond, (cudaGraphConditionalHandle)handle);
}

void launch_rebuild(const DevCtx& c, cudaStream_t s) {
    unsigned ga = grid_for(c.n);
    k_zero_cells<<<c.nsys, 256, 0, s>>>(c);
    if (c.nd == 3) k_bin<3><<<ga, BLOCK, 0, s>>>(c); else k_bin<2><<<ga, BLOCK, 0, s>>>(c);
    const uint32_t nblk = (c.nbucket + SCAN_CHUNK - 1) / SCAN_CHUNK;
    k_scan_blocks<<<nblk, SCAN_THREADS, 0, s>>>(c);
    k_scan_aux<<<1, SCAN_THREADS, 0, s>>>(c, nblk);
    k_scan_write<<<nblk, SCAN_THREADS, 0, s>>>(c);
    k_scatter<<<ga, BLOCK, 0, s>>>(c);
    k_cellsort<<<(unsigned)(((size_t)c.nbucket * 32 + BLOCK - 1) / BLOCK), BLOCK, 0, s>>>(c);
    if (c.staged) {
        if (c.nd == 3) {
            k_gather<3><<<ga, BLOCK, 0, s>>>(c);
            k_copyback<3><<<ga, BLOCK, 0, s>>>(c);
        } else {
            k_gather<2><<<ga, BLOCK, 0, s>>>(c);
            k_copyback<2><<<ga, BLOCK, 0, s>>>(c);
        }
        launch_build_stg(c, s);
        return;
    }
    if (c.any_lees) {   // FP64 handles only
        if (c.nd == 3) {
            k_gather<3><<<ga, BLOCK, 0, s>>>(c);
            k_copyback<3><<<ga, BLOCK, 0, s>>>(c);
            k_build_lees<3><<<ga, BLOCK, 0, s>>>(c);
        } else {
            k_gather<2><<<ga, BLOCK, 0, s>>>(c);
            k_copyback<2><<<ga, BLOCK, 0, s>>>(c);
            k_build_lees<2><<<ga, BLOCK, 0, s>>>(c);
        }
        k_sort_lists<<<grid_for(c.n, 128), 128, 0, s>>>(c);
        return;
    }
    if (c.nd == 3) {
        k_gather<3><<<ga, BLOCK, 0, s>>>(c);
        k_copyback<3><<<ga, BLOCK, 0, s>>>(c);
        if (c.any_wrap) k_build<3, true><<<(c.nbucket + BUILD_WARPS - 1) / BUILD_WARPS, BUILD_WARPS * 32, 0, s>>>(c);
        else k_build<3, false><<<(c.nbucket + BUILD_WARPS - 1) / BUILD_WARPS, BUILD_WARPS * 32, 0, s>>>(c);
    } else {
        k_gather<2><<<ga, BLOCK, 0, s>>>(c);
        k_copyback<2><<<ga, BLOCK, 0, s>>>(c);
        if (c.any_wrap) k_build<2, true><<<(c.nbucket + BUILD_WARPS - 1) / BUILD_WARPS, BUILD_WARPS * 32, 0, s>>>(c);
        else k_build<2, false><<<(c.nbucket + BUILD_WARPS - 1) / BUILD_WARPS, BUILD_WARPS * 32, 0, s>>>(c);
    }
    if (c.prec == PREC_FP64) {
        k_sort_lists<<<grid_for(c.n, 128), 128, 0, s>>>(c);
    } else if (c.ntile && c.tiled) {
        launch_tiles(c, s, 0);
    }
}

void launch_tiles(const DevCtx& c, cudaStream_t s, int all) {
    if (c.nd == 3) k_tile<3><<<c.ntile, TILE_ATOMS, 0, s>>>(c, all);
    else k_tile<2><<<c.ntile, TILE_ATOMS, 0, s>>>(c, all);
}

void launch_check(const DevCtx& c, cudaStream_t s) {
    if (c.nd == 3) k_check<3><<<grid_for(c.n), BLOCK, 0, s>>>(c);
    else k_check<2><<<grid_for(c.n), BLOCK, 0, s>>>(c);
}

void launch_numpairs(const DevCtx& c, cudaStream_t s) {
    k_count_half<<<grid_for(c.n), BLOCK, 0, s>>>(c);
}

void launch_reframe(const DevCtx& c, cudaStream_t s) {
    if (!c.rec) return;
    if (c.nd == 3) k_reframe<3><<<grid_for(c.n), BLOCK, 0, s>>>(c);
    else k_reframe<2><<<grid_for(c.n), BLOCK, 0, s>>>(c);
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
