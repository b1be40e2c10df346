// Mixed-precision cell-block kernels: list build, pair forces and list
// expansion with the neighbourhood of a block of cells staged in shared memory.
//
// Reference behaviour (wackywendell/parm): NeighborList::update_list
// (src/trackers.cpp:19-85) keeps every pair with
// |diff(x_i, x_j)| < (d_i + d_j)/2 + skin; NListed::set_forces
// (src/interaction.hpp:2165-2175) adds the pair force of every listed pair.
// The pair set here is the reference's exactly (FP32 screening, exact FP64
// test near the threshold); forces are FP32 sums, as in pair32.cu.
//
// Blocks.  A system whose cell grid has at least 3 cells along every axis is
// cut into blocks of Kx x Ky cells of one z layer (x fastest, the order of
// the cells in memory).  The block's neighbourhood is made of "rows": the
// cells x0-1 .. x1 of the y rows y0-1 .. y1 in the z layers z-1, z, z+1
// (2D: no z).  Each row is three "pieces" (left cell, the block's own cells,
// right cell), each a contiguous range of atoms in memory with one periodic
// image; pieces are numbered row by row and their atoms get consecutive local
// indices.  Kx <= nx - 2 and Ky <= ny - 2, so no atom appears twice in a
// block's neighbourhood.
//
// Staged record (16 bytes) of atom j: its cell-block record (kept per atom
// by the list build and the time-step kernels; parm_ctx.cuh) moved into the
// block's frame.  The block frame's origin is the lower edge of its first
// neighbour cell along each axis (on the 1/8 grid); a piece adds one packed
// constant K_p (its periodic shift and, along y and z, its row origin, in
// units of 1/8) to the coarse fields and its periodic shift's fine part
// s (L - L8) to the fine part.  Every staged field is then an exact integer
// 8 * (local position) + 256 within [0, 3840) (x, 12 bits) or [0, 768)
// (y, z, 10 bits), and a pair displacement is 0.125 * (q_i - q_j) +
// (f_i - f_j): the coarse difference is exact and only the fine parts round.
// One 32-bit subtraction (W_i + 256 per field) - W_j forms the three biased
// differences at once (each in [0, 2^bits) for atoms less than 32 apart, so
// no borrow crosses a field), and OR-ing a field into the mantissa of
// 1.5 * 2^20 (ulp 1/8) turns it into 1.5 * 2^20 + (q_i - q_j + 256) / 8
// exactly.
//
// The list build only screens candidates, so it stages plain FP32 positions
// relative to the centre of the block's neighbourhood (0.125 (q - c) + f, one
// rounding); pairs within 2e-5 (relative, on r^2) of the threshold are
// decided by the exact FP64 test.
//
// Lists.  Entries are 16-bit local indices.  The home atoms of a block are the
// atoms of its own pieces in the z = 0 layer (one contiguous range of memory
// per home row).  For a home row starting at atom s0 with H atoms, entry k of
// home atom s0 + h lives at u16 offset s0 * maxnb + (k / 2) * 2H + 2h + k % 2,
// so a warp reads the entries of 32 consecutive atoms as one coalesced line of
// 32-bit words (two entries each).
#include "parm_check.cuh"
#include "parm_pair32.cuh"

namespace parm {

constexpr int STG_THREADS = STG_THREADS_HOST;
constexpr float STG_BAND = 2e-5f;   // relative band on r^2 decided by the exact FP64 test
constexpr float CUT_BAND_S = 4e-6f; // LJ cut-off band (see pair32.cu)

struct __align__(16) StgTable {
    uint32_t g0[STG_PIECES_MAX];        // first atom of each piece
    uint32_t cnt[STG_PIECES_MAX];       // atoms in each piece
    uint32_t off[STG_PIECES_MAX + 1];   // local index of the first atom of each piece
    uint32_t K[STG_PIECES_MAX];         // packed coarse shift of each piece
    float F[STG_PIECES_MAX][3];         // fine part of each piece's periodic shift
    uint32_t rowbase[STG_ROWS_MAX];     // bucket of cell x = 0 of each row
    uint32_t hoff[STG_KY_MAX + 1];      // home atoms before each home row
    uint32_t hnmax[STG_KY_MAX];         // longest list of each home row (from the last build)
    int pc[3];                          // 256 + 8 * (neighbourhood centre) (plain positions)
    uint32_t nrow, npiece, total, nhome, nyr;
    int x0, x1, y0, y1, z;
};

static_assert(sizeof(StgTable) <= 16 * STG_TAB_WORDS, "block table larger than its slot");
constexpr uint32_t STG_TAB_USED = (uint32_t)((sizeof(StgTable) + 15) / 16);

__device__ __forceinline__ int wrap_idx(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

// The block tables depend on the cell arrays and the box only: the list
// build (and the list conversion) store them, the per-step kernels load them.
__device__ __forceinline__ void stg_store_table(const DevCtx& c, const StgTable& T, uint32_t b) {
    const float4* src = reinterpret_cast<const float4*>(&T);
    for (uint32_t t = threadIdx.x; t < STG_TAB_USED; t += blockDim.x)
        c.stg_tab[(size_t)b * STG_TAB_WORDS + t] = src[t];
}
// longest list of each home row (all threads; ends with a barrier)
template <int ND>
__device__ void stg_row_nmax(const DevCtx& c, StgTable& T) {
    for (uint32_t r = threadIdx.x; r < STG_KY_MAX; r += blockDim.x) T.hnmax[r] = 0u;
    __syncthreads();
    for (uint32_t h = threadIdx.x; h < T.nhome; h += blockDim.x) {
        uint32_t hr = 0;
        while (h >= T.hoff[hr + 1]) hr++;
        const uint32_t p = 3u * ((ND == 3 ? T.nyr : 0u) + hr + 1u) + 1u;
        atomicMax(&T.hnmax[hr], c.nnb[T.g0[p] + (h - T.hoff[hr])]);
    }
    __syncthreads();
}

__device__ __forceinline__ void stg_load_table(const DevCtx& c, StgTable& T, uint32_t b) {
    float4* dst = reinterpret_cast<float4*>(&T);
    for (uint32_t t = threadIdx.x; t < STG_TAB_USED; t += blockDim.x)
        dst[t] = __ldg(&c.stg_tab[(size_t)b * STG_TAB_WORDS + t]);
    __syncthreads();
}

// fill the block table (all threads; ends with a barrier)
template <int ND>
__device__ void stg_setup(const DevCtx& c, const SysConst& S, const uint4& bd, StgTable& T) {
    const int x0 = (int)(bd.y & 0xFFFFu), x1 = (int)(bd.y >> 16);
    const int y0 = (int)(bd.z & 0xFFFFu), y1 = (int)(bd.z >> 16);
    const int z = (int)bd.w;
    const int nyr = y1 - y0 + 2;
    const int nrow = (ND == 3 ? 3 : 1) * nyr;
    const int npiece = 3 * nrow;
    const uint32_t b0 = c.bucket_off[bd.x];
    const int nx = S.nc[0], ny = S.nc[1], nz = S.nc[2];
    // block frame origin (units of 1/8): lower edge of the first neighbour cell
    const int xb8 = rec_origin8(S, 0, x0 - 1), yb8 = rec_origin8(S, 1, y0 - 1);
    const int zb8 = (ND == 3) ? rec_origin8(S, 2, z - 1) : 0;
    // one thread per piece (row r = t / 3, part t % 3: left cell, the block's
    // cells, right cell)
    for (int t = threadIdx.x; t < npiece; t += blockDim.x) {
        const int r = t / 3, part = t % 3;
        const int dz = (ND == 3) ? r / nyr - 1 : 0;
        const int yy = y0 - 1 + r % nyr, zz = z + dz;
        const int cy = wrap_idx(yy, ny), cz = (ND == 3) ? wrap_idx(zz, nz) : 0;
        const uint32_t rb = b0 + (uint32_t)((cz * ny + cy) * nx);
        if (part == 0) T.rowbase[r] = rb;
        uint32_t lo, hi;
        int sx = 0;   // periodic shift of the piece along x (boxes)
        if (part == 0) {
            lo = rb + (uint32_t)wrap_idx(x0 - 1, nx);
            hi = lo + 1;
            sx = x0 == 0 ? -1 : 0;
        } else if (part == 1) {
            lo = rb + (uint32_t)x0;
            hi = rb + (uint32_t)x1;
        } else {
            lo = rb + (uint32_t)wrap_idx(x1, nx);
            hi = lo + 1;
            sx = x1 == nx ? 1 : 0;
        }
        const int sy = yy < 0 ? -1 : (yy >= ny ? 1 : 0);
        const int sz = (ND == 3) ? (zz < 0 ? -1 : (zz >= nz ? 1 : 0)) : 0;
        const uint32_t g = c.cell_start[lo];
        T.g0[t] = g;
        T.cnt[t] = c.cell_start[hi] - g;
        const int kx = sx * (int)(S.L8[0] * 8.0f) - xb8;
        const int ky = rec_origin8(S, 1, cy) + sy * (int)(S.L8[1] * 8.0f) - yb8;
        const int kz = (ND == 3) ? rec_origin8(S, 2, cz) + sz * (int)(S.L8[2] * 8.0f) - zb8 : 0;
        T.K[t] = (uint32_t)kx + ((uint32_t)ky << 12) + ((uint32_t)kz << 22);
        T.F[t][0] = (float)sx * S.Lr8[0];
        T.F[t][1] = (float)sy * S.Lr8[1];
        T.F[t][2] = (float)sz * S.Lr8[2];
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        // exclusive scan of the piece sizes, 32 pieces per pass
        const uint32_t lane = threadIdx.x;
        uint32_t carry = 0;
        for (int base = 0; base < npiece; base += 32) {
            const int p = base + (int)lane;
            const uint32_t v = p < npiece ? T.cnt[p] : 0u;
            uint32_t inc = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, inc, o);
                if (lane >= (uint32_t)o) inc += u;
            }
            if (p < npiece) T.off[p] = carry + inc - v;
            carry += __shfl_sync(0xFFFFFFFFu, inc, 31);
        }
        if (lane == 0) {
            T.off[npiece] = carry;
            T.total = carry;
            T.nrow = (uint32_t)nrow;
            T.npiece = (uint32_t)npiece;
            T.nyr = (uint32_t)nyr;
            T.x0 = x0; T.x1 = x1; T.y0 = y0; T.y1 = y1; T.z = z;
            const int hbase = (ND == 3) ? nyr : 0;   // first home row (z layer 0, y = y0)
            uint32_t h = 0;
            for (int hr = 0; hr < y1 - y0; hr++) {
                T.hoff[hr] = h;
                h += T.cnt[3 * (hbase + hr + 1) + 1];
            }
            T.hoff[y1 - y0] = h;
            for (int r = 0; r < STG_KY_MAX; r++) T.hnmax[r] = 0u;
            T.nhome = h;
            // centre of the neighbourhood in the block frame (plain positions)
            T.pc[0] = REC_BIAS + (int)rint(4.0 * (double)(x1 - x0 + 2) * S.cellw[0]);
            T.pc[1] = REC_BIAS + (int)rint(4.0 * (double)(y1 - y0 + 2) * S.cellw[1]);
            T.pc[2] = REC_BIAS + ((ND == 3) ? (int)rint(12.0 * S.cellw[2]) : 0);
        }
    }
    __syncthreads();
}

// cell-block record R of an atom of piece p, moved into the block frame
__device__ __forceinline__ float4 stg_shift(const StgTable& T, uint32_t p, const float4& R) {
    return make_float4(R.x + T.F[p][0], R.y + T.F[p][1], R.z + T.F[p][2],
                       __uint_as_float(__float_as_uint(R.w) + T.K[p]));
}

// one bulk request that brings [p, p + bytes) into L2 (16-byte aligned start
// and size); it completes on its own and nothing waits for it
__device__ __forceinline__ void prefetch_l2(const void* p, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// the records of the block's pieces (and, for the force kernel, the home
// rows' lists) requested into L2 at once, ahead of the staging loads
template <int ND>
__device__ __forceinline__ void stg_prefetch(const DevCtx& c, const StgTable& T, bool lists) {
    for (uint32_t t = threadIdx.x; t < T.npiece; t += blockDim.x)
        if (T.cnt[t]) prefetch_l2(c.rec + T.g0[t], T.cnt[t] * 16u);
    const uint32_t nhr = (uint32_t)(T.y1 - T.y0);
    if (lists && threadIdx.x >= 128u && threadIdx.x - 128u < nhr) {
        const uint32_t p = 3u * ((ND == 3 ? T.nyr : 0u) + (threadIdx.x - 128u) + 1u) + 1u;
        // the row's lists are word-major (word w of atom h at w * H + h), so
        // the words in use form a prefix; rows start 16-byte aligned (maxnb
        // is a multiple of 8) and the prefix is rounded up inside the row
        const uint32_t words = ((T.hnmax[threadIdx.x - 128u] + 1u) >> 1) * T.cnt[p];
        const uint32_t bytes = min((words * 4u + 15u) & ~15u, T.cnt[p] * c.maxnb * 2u);
        if (bytes) prefetch_l2(c.nbr16 + (size_t)T.g0[p] * c.maxnb, bytes);
    }
}

// piece of local index q (binary search over the offsets)
__device__ __forceinline__ uint32_t stg_piece(const StgTable& T, uint32_t q) {
    uint32_t lo = 0, hi = T.npiece;   // off[lo] <= q < off[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (T.off[mid] <= q) lo = mid; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ uint32_t stg_global(const StgTable& T, uint32_t q) {
    const uint32_t p = stg_piece(T, q);
    return T.g0[p] + (q - T.off[p]);
}

// a local index that does not belong to the block (inconsistent lists) is
// reported and replaced by the home atom itself, whose pair term is zero
__device__ __forceinline__ uint32_t stg_check(const DevCtx& c, const StgTable& T, uint32_t q, uint32_t qi) {
    if (q < T.total) return q;
    atomicOr(c.status, ST_TILE_OVERFLOW);
    return qi;
}

// record of local index q: shared memory, or rebuilt from global memory when
// the neighbourhood is larger than the staging capacity
template <int ND>
__device__ __forceinline__ float4 stg_get(const DevCtx& c, const SysConst& S, const StgTable& T,
                                          const float4* srec, uint32_t cap, uint32_t q) {
    if (q < cap) return srec[q];
    const uint32_t p = stg_piece(T, q);
    return stg_shift(T, p, c.rec[T.g0[p] + (q - T.off[p])]);
}

constexpr uint32_t STG_GUARD = 256u | (256u << 12) | (256u << 22);   // + 256 per field
constexpr uint32_t STG_MANT = 0x49C00000u;                           // 1.5 * 2^20, ulp 1/8
constexpr float STG_K = 1572864.0f + 32.0f;                          // 1.5 * 2^20 + 256 / 8

// W_i + 256 per field (the home atom's side of the packed subtraction)
__device__ __forceinline__ uint32_t stg_wi(const float4& ri) { return __float_as_uint(ri.w) + STG_GUARD; }

// displacement x_i - x_j from two packed records
template <int ND>
__device__ __forceinline__ void stg_disp(uint32_t wi, const float4& ri, const float4& rj, float* r) {
    const uint32_t D = wi - __float_as_uint(rj.w);
    r[0] = (__uint_as_float((D & 0xFFFu) | STG_MANT) - STG_K) + (ri.x - rj.x);
    r[1] = (__uint_as_float(((D >> 12) & 0x3FFu) | STG_MANT) - STG_K) + (ri.y - rj.y);
    if constexpr (ND == 3) r[2] = (__uint_as_float((D >> 22) | STG_MANT) - STG_K) + (ri.z - rj.z);
    else r[2] = 0.f;
}

// plain FP32 position relative to the neighbourhood centre (list screening)
__device__ __forceinline__ float4 stg_plain(const StgTable& T, const float4& rec, float w) {
    const uint32_t W = __float_as_uint(rec.w);
    const float qx = (float)((int)(W & 0xFFFu) - T.pc[0]), qy = (float)((int)((W >> 12) & 0x3FFu) - T.pc[1]),
                qz = (float)((int)(W >> 22) - T.pc[2]);
    return make_float4(fmaf(qx, 0.125f, rec.x), fmaf(qy, 0.125f, rec.y), fmaf(qz, 0.125f, rec.z), w);
}

// The plain stage is pair-interleaved: local indices 2k and 2k + 1 share 32
// bytes, (x0, x1, y0, y1) then (z0, z1, w0, w1), so one 16-byte load gives the
// x and y of two candidates as packed FP32 pairs.
__device__ __forceinline__ void stg_put_plain(float4* sp, uint32_t q, const float4& v) {
    float* f = reinterpret_cast<float*>(sp) + 8u * (q >> 1) + (q & 1u);
    f[0] = v.x;
    f[2] = v.y;
    f[4] = v.z;
    f[6] = v.w;
}
__device__ __forceinline__ float4 stg_at_plain(const float4* sp, uint32_t q) {
    const float* f = reinterpret_cast<const float*>(sp) + 8u * (q >> 1) + (q & 1u);
    return make_float4(f[0], f[2], f[4], f[6]);
}

// list diameter of atom j (the w of its coarse position view)
__device__ __forceinline__ float stg_diam(const DevCtx& c, uint32_t j) {
    return __ldg(reinterpret_cast<const float*>(c.pos + 2 * (size_t)j) + 3);
}

// Staging for the list build: plain FP32 positions of the first `cap` local
// indices (w: the list diameter when `diam`, else 0), warp per piece.  Each
// warp takes two pieces at a time and each lane issues the loads of up to
// four atoms (two per piece) before converting any, so that their latencies
// overlap.
__device__ void stg_load_plain(const DevCtx& c, const StgTable& T, float4* sp, uint32_t cap, bool diam) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (uint32_t p0 = warp; p0 < T.npiece; p0 += 2 * nw) {
        float4 R[4];
        float w[4];
        uint32_t q[4], pc[4];
        bool ok[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const uint32_t p = p0 + (k >> 1) * nw;
            const uint32_t t = lane + 32u * (k & 1);
            pc[k] = p;
            ok[k] = p < T.npiece && t < T.cnt[p] && T.off[p] + t < cap;
            q[k] = ok[k] ? T.off[p] + t : 0u;
            w[k] = 0.f;
            if (ok[k]) {
                const uint32_t j = T.g0[p] + t;
                R[k] = __ldg(&c.rec[j]);
                if (diam) w[k] = stg_diam(c, j);
            }
        }
#pragma unroll
        for (int k = 0; k < 4; k++)
            if (ok[k]) stg_put_plain(sp, q[k], stg_plain(T, stg_shift(T, pc[k], R[k]), w[k]));
        // pieces longer than 64 atoms (large blocks of sparse systems)
#pragma unroll 1
        for (int k = 0; k < 2; k++) {
            const uint32_t p = p0 + k * nw;
            if (p >= T.npiece) break;
            for (uint32_t t = lane + 64u; t < T.cnt[p] && T.off[p] + t < cap; t += 32u) {
                const uint32_t j = T.g0[p] + t;
                stg_put_plain(sp, T.off[p] + t, stg_plain(T, stg_shift(T, p, __ldg(&c.rec[j])), diam ? stg_diam(c, j) : 0.f));
            }
        }
    }
    __syncthreads();
}

// ---- bulk (TMA) staging: one asynchronous copy per piece into shared memory,
// completion counted in bytes on one mbarrier ----
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
// waits for phase 0 of the barrier, at most `limit` polls; false on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t limit) {
    for (uint32_t it = 0; it < limit; it++) {
        uint32_t done;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(smem_addr(bar)), "r"(0u)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Staging by bulk copies: every piece's records (and, EXTRA == 2, its FP32
// pair parameters) are copied into shared memory as they lie in global
// memory (one asynchronous copy per piece, 16-byte aligned, completion
// counted on one mbarrier), then each warp moves its pieces' records into
// the block frame in place.  Returns false (and flags ST_STAGE_TIMEOUT) when
// the copies do not complete within the wait limit; if they are still not
// complete after a second bounded wait, no thread touches the staged shared
// memory again.
template <int ND, int EXTRA>
__device__ bool stg_load_bulk(const DevCtx& c, const StgTable& T, float4* srec, void* sext, uint32_t cap,
                              uint64_t* bar) {
    const uint32_t staged = min(T.total, cap);
    const uint32_t per = (EXTRA == 2) ? 32u : 16u;
    if (threadIdx.x == 0) mbar_init(bar, 1);
    __syncthreads();
    if (threadIdx.x == 0) mbar_arrive_tx(bar, staged * per);
    for (uint32_t p = threadIdx.x; p < T.npiece; p += blockDim.x) {
        const uint32_t o = T.off[p];
        if (o >= cap || T.cnt[p] == 0) continue;
        const uint32_t n = min(T.cnt[p], cap - o);
        bulk_g2s(srec + o, c.rec + T.g0[p], n * 16u, bar);
        if constexpr (EXTRA == 2) bulk_g2s(static_cast<float4*>(sext) + o, c.prm32 + T.g0[p], n * 16u, bar);
    }
    const bool ok = mbar_wait(bar, 1u << 22);
    bool settled = ok;
    if (!ok) {
        atomicOr(c.status, ST_STAGE_TIMEOUT);
        settled = mbar_wait(bar, 1u << 22);   // the copies in flight, once more with a limit
    }
    // unless every thread saw the copies complete, the block leaves its
    // shared memory alone (no rewrite, no pair loop) and returns at once
    if (!__syncthreads_and(settled)) return false;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (uint32_t p = warp; p < T.npiece; p += nw) {
        const uint32_t o = T.off[p];
        if (o >= cap) continue;
        const uint32_t n = min(T.cnt[p], cap - o);
        const uint32_t K = T.K[p];
        const float F0 = T.F[p][0], F1 = T.F[p][1], F2 = T.F[p][2];
        for (uint32_t t = lane; t < n; t += 32u) {
            float4 r = srec[o + t];
            r.x += F0;
            r.y += F1;
            r.z += F2;
            r.w = __uint_as_float(__float_as_uint(r.w) + K);
            srec[o + t] = r;
            if constexpr (EXTRA == 1) static_cast<float*>(sext)[o + t] = __ldg(&c.prm32[T.g0[p] + t].y);
        }
    }
    return __syncthreads_and(ok) != 0;   // the same answer in every thread
}

// home atom h -> (home row, global atom, local index, cell x)
struct HomeAtom {
    uint32_t hr, i, qi, s0, H, hs;
    int cx;
};

template <int ND, bool CELL = true>
__device__ __forceinline__ HomeAtom stg_home(const DevCtx& c, const StgTable& T, uint32_t h) {
    HomeAtom a;
    uint32_t hr = 0;
    while (h >= T.hoff[hr + 1]) hr++;
    const uint32_t r = (ND == 3 ? T.nyr : 0u) + hr + 1u;
    const uint32_t p = 3u * r + 1u;
    a.hr = hr;
    a.hs = h - T.hoff[hr];
    a.s0 = T.g0[p];
    a.H = T.cnt[p];
    a.i = a.s0 + a.hs;
    a.qi = T.off[p] + a.hs;
    a.cx = T.x0;
    if constexpr (CELL) {
        a.cx = (int)(c.bucket[a.i] - T.rowbase[r]);
        if (a.cx < T.x0 || a.cx >= T.x1) {   // never for lists of the current grid
            atomicOr(c.status, ST_CELL_RANGE);
            a.cx = T.x0;
        }
    }
    return a;
}

// local candidate range of a home atom in stencil row r
__device__ __forceinline__ void stg_range(const DevCtx& c, const StgTable& T, uint32_t r, int cx,
                                          uint32_t& lo, uint32_t& hi) {
    const uint32_t pm = 3u * r + 1u;
    lo = (cx == T.x0) ? T.off[pm - 1] : T.off[pm] + (c.cell_start[T.rowbase[r] + (uint32_t)(cx - 1)] - T.g0[pm]);
    hi = (cx == T.x1 - 1) ? T.off[pm + 1] + T.cnt[pm + 1]   // through the right piece
                          : T.off[pm] + (c.cell_start[T.rowbase[r] + (uint32_t)(cx + 2)] - T.g0[pm]);
}

__device__ __forceinline__ size_t stg_entry16(const HomeAtom& a, uint32_t maxnb, uint32_t k) {
    return (size_t)a.s0 * maxnb + (size_t)(k >> 1) * 2u * a.H + 2u * a.hs + (k & 1u);
}

// exact reference list test, explicit round-to-nearest FP64 operations:
// diff(x_i, x_j).norm() < (d_i + d_j)/2 + skin
template <int ND>
__device__ __noinline__ bool keep_exact_rn(const DevCtx& c, const SysConst& S, uint32_t i, uint32_t j) {
    const double* a = reinterpret_cast<const double*>(c.x) + (size_t)i * (ND == 3 ? 4 : 2);
    const double* b = reinterpret_cast<const double*>(c.x) + (size_t)j * (ND == 3 ? 4 : 2);
    double sq[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int d = 0; d < ND; d++) {
        const double r = remainder_exact(__dsub_rn(a[d], b[d]), S.L[d], S.invL[d], S.halfL[d]);
        sq[d] = __dmul_rn(r, r);
    }
    double s2 = __dadd_rn(sq[0], sq[1]);
    if constexpr (ND == 3) s2 = __dadd_rn(s2, sq[2]);
    const double diam = __dmul_rn(__dadd_rn(c.diam[i], c.diam[j]), 0.5);
    return __dsqrt_rn(s2) < __dadd_rn(diam, S.skin);
}

__device__ __forceinline__ bool is_excluded_s(const DevCtx& c, uint32_t oi, uint32_t oj) {
    for (uint32_t e = c.excl_off[oi]; e < c.excl_off[oi + 1]; e++)
        if (c.excl_list[e] == oj) return true;
    return false;
}

// exact LJ cut-off classification (as lj_beyond_exact in pair32.cu)
__device__ __noinline__ bool lj_beyond_exact_s(const DevCtx& c, const SysConst& S, uint32_t i, uint32_t j,
                                               int nd) {
    const double* xi = reinterpret_cast<const double*>(c.x) + (size_t)i * (nd == 3 ? 4 : 2);
    const double* xj = reinterpret_cast<const double*>(c.x) + (size_t)j * (nd == 3 ? 4 : 2);
    double sq[3] = {0.0, 0.0, 0.0};
    for (int d = 0; d < nd; d++) {
        double r = remainder_exact(__dsub_rn(xi[d], xj[d]), S.L[d], S.invL[d], S.halfL[d]);
        sq[d] = __dmul_rn(r, r);
    }
    double dsq = __dadd_rn(sq[0], sq[1]);
    if (nd == 3) dsq = __dadd_rn(dsq, sq[2]);
    const AtomPrm A = c.prm[i], B = c.prm[j];
    const double sig = __dmul_rn(__dadd_rn(A.p1, B.p1), 0.5);
    const double cut = B.p2 > A.p2 ? B.p2 : A.p2;
    const double rsq = __ddiv_rn(dsq, __dmul_rn(sig, sig));
    return rsq > __dmul_rn(cut, cut);
}

// non-member atoms of a system (no neighbours, zero force)
__device__ void stg_nonmembers(const DevCtx& c, uint32_t s, int zero_a) {
    const SysConst& S = c.sys[s];
    const uint32_t b = c.bucket_off[s] + S.ncell;
    const uint32_t hi = S.atom_off + S.natoms;
    const uint32_t lo = max(c.cell_start[b], S.atom_off);
    for (uint32_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        c.nnb[i] = 0u;
        c.f32[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (zero_a) {
            double* a = static_cast<double*>(c.a) + (size_t)i * (c.nd == 3 ? 4 : 2);
            for (int d = 0; d < c.nd; d++) a[d] = 0.0;
        }
    }
}

__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// packed pairs of FP32 values (Blackwell's f32x2 add / mul / fma: two lanes
// of work per instruction)
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 pk2(float a, float b) {
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void upk2(f32x2 r, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ f32x2 add2(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 sub2(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 mul2(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c) {
    f32x2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

// ---------------------------------------------------------------------------
// list build: one CTA per block, one thread per home atom
// ---------------------------------------------------------------------------
// plain position of local index q; w: the list diameter (DIA) or 0
template <int ND, int DIA>
__device__ __forceinline__ float4 stg_get_plain(const DevCtx& c, const SysConst& S, const StgTable& T,
                                                const float4* sp, uint32_t cap, uint32_t q) {
    if (q < cap) return stg_at_plain(sp, q);
    const uint32_t p = stg_piece(T, q);
    const uint32_t j = T.g0[p] + (q - T.off[p]);
    return stg_plain(T, stg_shift(T, p, c.rec[j]), DIA ? stg_diam(c, j) : 0.f);
}

template <int ND, int DIA, bool FULL>
__device__ __forceinline__ void build_home(const DevCtx& c, const SysConst& S, const StgTable& T,
                                           const float4* sp, uint32_t cap, const HomeAtom& a) {
    const uint32_t maxnb = c.maxnb;
    uint16_t* out = c.nbr16;
    const float skin32 = (float)S.skin;
    const float4 P = FULL ? stg_at_plain(sp, a.qi) : stg_get_plain<ND, DIA>(c, S, T, sp, cap, a.qi);
    const float tu = (DIA ? P.w : stg_diam(c, a.i)) + skin32;
    const float hiu = tu * tu * (1.0f + STG_BAND), lou = tu * tu * (1.0f - STG_BAND);
    const uint32_t oi = c.excl_off ? c.orig[a.i] : 0u;
    // entry k of this atom: ob[(k / 2) * 2H + k % 2], i.e. half k % 2 of the
    // 32-bit word ow[(k / 2) * H] (maxnb is a multiple of 8)
    uint16_t* const ob = out + (size_t)a.s0 * maxnb + 2u * a.hs;
    uint32_t* const ow = reinterpret_cast<uint32_t*>(ob);
    const uint32_t H2 = 2u * a.H;
    uint32_t k = 0, pend = 0u;
    // broadcast pairs for the packed screening of FULL stages
    const f32x2 Px2 = pk2(P.x, P.x), Py2 = pk2(P.y, P.y), Pz2 = pk2(P.z, P.z);
    const f32x2 HI2 = pk2(hiu, hiu), LO2 = pk2(lou, lou);
    const f32x2 PW2 = pk2(P.w, P.w), HALF2 = pk2(0.5f, 0.5f), SKIN2 = pk2(skin32, skin32);
    const f32x2 BH2 = pk2(1.0f + STG_BAND, 1.0f + STG_BAND), BL2 = pk2(1.0f - STG_BAND, 1.0f - STG_BAND);
#pragma unroll 1
    for (int dz = 0; dz < (ND == 3 ? 3 : 1); dz++) {
#pragma unroll 1
        for (int dy = 0; dy < 3; dy++) {
            const uint32_t r = (uint32_t)dz * T.nyr + a.hr + (uint32_t)dy;
            uint32_t lo, hi;
            stg_range(c, T, r, a.cx, lo, hi);
            // 32 candidates at a time: a branch-free screening pass sets one
            // bit per candidate within the widened threshold, then the set
            // bits (the ~15 % that are kept) are settled and written in order
#pragma unroll 1
            // FULL stages are screened two candidates at a time in packed
            // FP32 pairs, so the passes start at an even local index (an odd
            // row start adds the slot before it, cleared below)
            for (uint32_t base = FULL ? (lo & ~1u) : lo; base < hi; base += 32u) {
                const uint32_t m = min(32u, hi - base);
                uint32_t mask = 0u, sure = 0u;
                // bit of a candidate within the widened threshold (mask) and
                // within the narrowed one (sure: kept without the exact test)
                auto screen = [&](const float4& Q, uint32_t bit) {
                    const float dx = P.x - Q.x, dyv = P.y - Q.y;
                    float rr = fmaf(dyv, dyv, dx * dx);
                    if constexpr (ND == 3) {
                        const float dzv = P.z - Q.z;
                        rr = fmaf(dzv, dzv, rr);
                    }
                    float hi2 = hiu, lo2 = lou;
                    if constexpr (DIA) {
                        const float thr = 0.5f * (P.w + Q.w) + skin32;
                        hi2 = thr * thr * (1.0f + STG_BAND);
                        lo2 = thr * thr * (1.0f - STG_BAND);
                    }
                    mask |= rr <= hi2 ? bit : 0u;
                    sure |= rr < lo2 ? bit : 0u;
                };
                if constexpr (FULL) {
                    // all 32 slots (the stage has 32 records of padding past
                    // its capacity), then the slots past the row, the slot
                    // before an odd row start and the home atom itself are
                    // cleared.  A candidate's bit is the sign of rr - hi2
                    // (rr < hi2; equality is far outside the true threshold,
                    // which lies 2e-5 below hi2) and of rr - lo2 (rr < lo2),
                    // shifted in from the top candidate down so that bit u
                    // is candidate base + u.
                    const ulonglong2* sq = reinterpret_cast<const ulonglong2*>(sp) + base;
#pragma unroll
                    for (int u2 = 15; u2 >= 0; u2--) {
                        const ulonglong2 A = sq[2 * u2];   // (x0, x1), (y0, y1)
                        const f32x2 dx = sub2(Px2, A.x), dy = sub2(Py2, A.y);
                        f32x2 rr = fma2(dy, dy, mul2(dx, dx));
                        f32x2 h2 = HI2, l2 = LO2;
                        if constexpr (ND == 3 || DIA) {
                            const ulonglong2 B = sq[2 * u2 + 1];   // (z0, z1), (w0, w1)
                            if constexpr (ND == 3) {
                                const f32x2 dz = sub2(Pz2, B.x);
                                rr = fma2(dz, dz, rr);
                            }
                            if constexpr (DIA) {
                                const f32x2 thr = fma2(add2(PW2, B.y), HALF2, SKIN2);
                                const f32x2 t2 = mul2(thr, thr);
                                h2 = mul2(t2, BH2);
                                l2 = mul2(t2, BL2);
                            }
                        }
                        float e0, e1, g0, g1;
                        upk2(sub2(rr, h2), e0, e1);
                        upk2(sub2(rr, l2), g0, g1);
                        mask = __funnelshift_l(__float_as_uint(e1), mask, 1);
                        sure = __funnelshift_l(__float_as_uint(g1), sure, 1);
                        mask = __funnelshift_l(__float_as_uint(e0), mask, 1);
                        sure = __funnelshift_l(__float_as_uint(g0), sure, 1);
                    }
                    if (m < 32u) mask &= (1u << m) - 1u;
                    if (base < lo) mask &= ~1u;
                    const uint32_t d = a.qi - base;
                    if (d < 32u) mask &= ~(1u << d);
                } else {
#pragma unroll 8
                    for (uint32_t u = 0; u < m; u++) {
                        const uint32_t q = base + u;
                        if (q != a.qi) screen(stg_get_plain<ND, DIA>(c, S, T, sp, cap, q), 1u << u);
                    }
                }
                // entries are written as 32-bit words of two (the even one
                // waits in `pend`)
                if ((mask & ~sure) == 0u && !c.excl_off) {
                    while (mask) {   // all kept
                        const uint32_t q = base + (uint32_t)__ffs(mask) - 1u;
                        mask &= mask - 1u;
                        if (k < maxnb) {
                            if (k & 1u) ow[(size_t)(k >> 1) * a.H] = pend | (q << 16);
                            else pend = q;
                        }
                        k++;
                    }
                    continue;
                }
                while (mask) {
                    const uint32_t u = (uint32_t)__ffs(mask) - 1u;
                    mask &= mask - 1u;
                    const uint32_t q = base + u;
                    bool keep = (sure >> u) & 1u;
                    uint32_t j = 0xFFFFFFFFu;
                    if (!keep) {   // rare: the exact reference test
                        j = stg_global(T, q);
                        keep = keep_exact_rn<ND>(c, S, a.i, j);
                    }
                    if (keep && c.excl_off) {
                        if (j == 0xFFFFFFFFu) j = stg_global(T, q);
                        keep = !is_excluded_s(c, oi, c.orig[j]);
                    }
                    if (!keep) continue;
                    if (k < maxnb) {
                        if (k & 1u) ow[(size_t)(k >> 1) * a.H] = pend | (q << 16);
                        else pend = q;
                    }
                    k++;
                }
            }
        }
    }
    {
        const uint32_t kk = min(k, maxnb);
        if (kk & 1u) ob[(size_t)(kk >> 1) * H2] = (uint16_t)pend;   // the last, unpaired entry
    }
    if (k > maxnb) {
        atomicOr(c.status, ST_NBR_OVERFLOW);
        k = maxnb;
    }
    c.nnb[a.i] = k;
    atomicMax(const_cast<uint32_t*>(&T.hnmax[a.hr]), k);
}

template <int ND, int DIA>
__global__ void __launch_bounds__(STG_THREADS, 4) k_build_stg(DevCtx c) {
    extern __shared__ float4 smem_b[];
    __shared__ StgTable T;
    if (blockIdx.x >= c.nblk) {
        const uint32_t s = blockIdx.x - c.nblk;
        if (c.flag[s]) stg_nonmembers(c, s, 0);
        return;
    }
    const uint4 bd = c.blk[blockIdx.x];
    if (!c.flag[bd.x]) return;
    const SysConst& S = c.sys[bd.x];
    stg_setup<ND>(c, S, bd, T);
    stg_prefetch<ND>(c, T, false);
    if (T.total > 0xFFFFu) {   // more than 65535 atoms around one block
        if (threadIdx.x == 0) atomicOr(c.status, ST_TILE_OVERFLOW);
        return;
    }
    const uint32_t cap = c.stg_cap;
    stg_load_plain(c, T, smem_b, cap, DIA != 0);
    const bool full = T.total <= cap;
    for (uint32_t h = threadIdx.x; h < T.nhome; h += blockDim.x) {
        const HomeAtom a = stg_home<ND>(c, T, h);
        if (full) build_home<ND, DIA, true>(c, S, T, smem_b, cap, a);
        else build_home<ND, DIA, false>(c, S, T, smem_b, cap, a);
    }
    __syncthreads();   // the home rows' longest lists are in the table now
    stg_store_table(c, T, blockIdx.x);
}

// ---------------------------------------------------------------------------
// pair forces: one CTA per block, one thread per home atom.  PRM: 0 uniform
// parameters, 1 per-atom sigma (epsilon and exponent / cut-off uniform),
// 2 per-atom (sqrt(eps), sigma, third).  A launch loads the block's table
// (stored by the list build), requests the pieces' records and the used part
// of the home rows' lists into L2, copies the records into shared memory with
// one bulk asynchronous copy per piece and moves them into the block frame.
// ---------------------------------------------------------------------------
// pair-law constants of one pair type
template <int KIND>
struct Law {
    float e12, isig2, sig, third, C, cut2, band;
    __device__ __forceinline__ void set(float e12_, float sig_, float isig2_, float third_) {
        e12 = e12_;
        sig = sig_;
        isig2 = isig2_;
        third = third_;
        C = e12 * isig2;
        cut2 = (KIND == KIND_LJCUT) ? third * third : 1.0f;
        band = CUT_BAND_S * cut2;
    }
    // LJ kinds: the force scale s (F_i += r * s) ignoring the cut-off, and
    // dd = r^2/sigma^2 - cut^2
    __device__ __forceinline__ float lj_raw(float d2, float& dd) const {
        const float rsq = d2 * isig2;
        const float ir = rcp_approx(rsq);
        const float ir2 = ir * ir;
        const float ir4 = ir2 * ir2;
        const float ir3 = ir2 * ir;
        const float t = C * ir4;
        dd = rsq - cut2;
        return fmaf(t, ir3, -t);   // 12 eps / sigma^2 * ir^4 (ir^3 - 1)
    }
    // force scale s (F_i += r * s), zero beyond the FP32 cut-off test; for
    // LJCUT, `dmin` tracks min(|dd| - band): a pair with |dd| <= band is
    // settled afterwards by the exact FP64 test
    __device__ __forceinline__ float scale(float d2, float& dmin) const {
        if constexpr (KIND == KIND_LJCUT || KIND == KIND_LJREPULSE) {
            float dd;
            const float sc = lj_raw(d2, dd);
            if constexpr (KIND == KIND_LJCUT) dmin = fminf(dmin, fabsf(dd) - band);
            return dd > 0.0f ? 0.0f : sc;
        } else {
            bool nc;
            return scale32<KIND>(d2, e12, sig, isig2, third, nc);
        }
    }
};

// per-home-atom data loaded from global memory before the pair loop (issued
// ahead of the staging wait for a thread's first home atom)
struct HomePre {
    uint32_t nn, w0, w1;
    float4 Qi;   // (sqrt(eps), sigma, third, m6)
    const uint32_t* row;
};

__device__ __forceinline__ HomePre home_pre(const DevCtx& c, const HomeAtom& a) {
    HomePre p;
    p.nn = c.nnb[a.i];
    p.Qi = c.prm32[a.i];
    p.row = reinterpret_cast<const uint32_t*>(c.nbr16) + ((size_t)a.s0 * c.maxnb >> 1) + a.hs;
    p.w0 = __ldg(p.row);       // entries of the first two words (read even when
    p.w1 = __ldg(p.row + a.H); // the list is shorter: they lie inside its region)
    return p;
}

template <int ND, int KIND, int PRM, bool FULL>
__device__ __forceinline__ void force_home(const DevCtx& c, const SysConst& S, const StgTable& T,
                                           const float4* srec, const void* sext, uint32_t cap,
                                           const HomeAtom& a, const HomePre& pre, const Law<KIND>& law0,
                                           float* f, uint32_t hidx) {
    float dmin = 1.0f;   // min over pairs of |rsq - cut^2| - band (LJCUT)
    const float4 ri = FULL ? srec[a.qi] : stg_get<ND>(c, S, T, srec, cap, a.qi);
    const uint32_t wi = stg_wi(ri);
    const float* ssig = static_cast<const float*>(sext);
    const float4* sprm = static_cast<const float4*>(sext);
    const float4 Qi = pre.Qi;
    const uint32_t nn = pre.nn;
    const uint32_t H = a.H;
    const uint32_t* row = pre.row;
    const uint32_t qmax = T.total - 1u;
    auto pair = [&](uint32_t q) {
        float4 rj;
        if (FULL) {
            q = min(q, qmax);
            rj = srec[q];
        } else {
            q = stg_check(c, T, q, a.qi);
            if (q == a.qi) return;
            rj = stg_get<ND>(c, S, T, srec, cap, q);
        }
        float r[3];
        stg_disp<ND>(wi, ri, rj, r);
        float d2 = fmaf(r[1], r[1], r[0] * r[0]);
        if constexpr (ND == 3) d2 = fmaf(r[2], r[2], d2);
        Law<KIND> law = law0;
        if constexpr (PRM == 1) {
            const float sj = (FULL || q < cap) ? ssig[q] : c.prm32[stg_global(T, q)].y;
            const float sg = 0.5f * (Qi.y + sj);
            law.set(law0.e12, sg, rcp_approx(sg * sg), law0.third);
        } else if constexpr (PRM == 2) {
            const float4 Qj = (FULL || q < cap) ? sprm[q] : c.prm32[stg_global(T, q)];
            const float eps = Qi.x * Qj.x;
            const float sg = 0.5f * (Qi.y + Qj.y);
            law.set((KIND == KIND_REPULSION) ? eps : 12.0f * eps, sg, rcp_approx(sg * sg),
                    (KIND == KIND_LJCUT) ? fmaxf(Qi.z, Qj.z) : 0.5f * (Qi.z + Qj.z));
        }
        const float sc = law.scale(d2, dmin);
#pragma unroll
        for (int d = 0; d < ND; d++) f[d] = fmaf(r[d], sc, f[d]);
    };
    const uint32_t nw = nn >> 1;   // words holding two entries
    uint32_t p = 0;
    if constexpr (FULL && PRM == 0 && (KIND == KIND_LJCUT || KIND == KIND_LJREPULSE)) {
        // the two entries of each list word together, in packed FP32 pairs:
        // even entries accumulate in the low half, odd ones in the high half
        const f32x2 K2 = pk2(STG_K, STG_K), is2 = pk2(law0.isig2, law0.isig2), C2 = pk2(law0.C, law0.C);
        const f32x2 P1_2 = pk2(1.0f, 1.0f);
        f32x2 fx = pk2(0.f, 0.f), fy = fx, fz = fx;
        auto pair2 = [&](uint32_t w) {
            const uint32_t q0 = min(w & 0xFFFFu, qmax), q1 = min(w >> 16, qmax);
            const float4 ra = srec[q0], rb = srec[q1];
            const uint32_t D0 = wi - __float_as_uint(ra.w), D1 = wi - __float_as_uint(rb.w);
            const f32x2 rx = add2(sub2(pk2(__uint_as_float((D0 & 0xFFFu) | STG_MANT),
                                           __uint_as_float((D1 & 0xFFFu) | STG_MANT)), K2),
                                  pk2(ri.x - ra.x, ri.x - rb.x));
            const f32x2 ry = add2(sub2(pk2(__uint_as_float(((D0 >> 12) & 0x3FFu) | STG_MANT),
                                           __uint_as_float(((D1 >> 12) & 0x3FFu) | STG_MANT)), K2),
                                  pk2(ri.y - ra.y, ri.y - rb.y));
            f32x2 d2 = fma2(ry, ry, mul2(rx, rx));
            f32x2 rz = pk2(0.f, 0.f);
            if constexpr (ND == 3) {
                rz = add2(sub2(pk2(__uint_as_float((D0 >> 22) | STG_MANT), __uint_as_float((D1 >> 22) | STG_MANT)),
                               K2),
                          pk2(ri.z - ra.z, ri.z - rb.z));
                d2 = fma2(rz, rz, d2);
            }
            float r0, r1;
            upk2(mul2(d2, is2), r0, r1);
            const f32x2 ir = pk2(rcp_approx(r0), rcp_approx(r1));
            const f32x2 ir2 = mul2(ir, ir);
            const f32x2 ir4 = mul2(ir2, ir2);
            const f32x2 ir3 = mul2(ir2, ir);
            const f32x2 t = mul2(C2, ir4);
            float s0, s1;
            // 12 eps / sigma^2 * ir^4 (ir^3 - 1); ir^3 - 1 is exact for ir^3 in
            // [1/2, 2] (the strongly repulsive and the attractive well's pairs),
            // so the product is the only rounding there
            upk2(mul2(t, sub2(ir3, P1_2)), s0, s1);
            const float dd0 = r0 - law0.cut2, dd1 = r1 - law0.cut2;
            if constexpr (KIND == KIND_LJCUT) dmin = fminf(dmin, fminf(fabsf(dd0), fabsf(dd1)) - law0.band);
            const f32x2 sc = pk2(dd0 > 0.0f ? 0.0f : s0, dd1 > 0.0f ? 0.0f : s1);
            fx = fma2(rx, sc, fx);
            fy = fma2(ry, sc, fy);
            if constexpr (ND == 3) fz = fma2(rz, sc, fz);
        };
        if (nw >= 2) {
            uint32_t w0 = pre.w0, w1 = pre.w1;
#pragma unroll 1
            for (; p + 3 < nw; p += 2) {
                const uint32_t n0 = __ldg(row + (size_t)(p + 2) * H), n1 = __ldg(row + (size_t)(p + 3) * H);
                pair2(w0);
                pair2(w1);
                w0 = n0;
                w1 = n1;
            }
            pair2(w0);
            pair2(w1);
            p += 2;
        }
        if (p < nw) pair2(p == 0 ? pre.w0 : __ldg(row + (size_t)p * H));
        float a0, a1;
        upk2(fx, a0, a1);
        f[0] = a0 + a1;
        upk2(fy, a0, a1);
        f[1] = a0 + a1;
        if constexpr (ND == 3) {
            upk2(fz, a0, a1);
            f[2] = a0 + a1;
        }
        p = nw;
    }
    if (nw >= 2 && p == 0) {
        uint32_t w0 = pre.w0, w1 = pre.w1;
#pragma unroll 1
        for (; p + 3 < nw; p += 2) {
            const uint32_t n0 = __ldg(row + (size_t)(p + 2) * H), n1 = __ldg(row + (size_t)(p + 3) * H);
            pair(w0 & 0xFFFFu);
            pair(w0 >> 16);
            pair(w1 & 0xFFFFu);
            pair(w1 >> 16);
            w0 = n0;
            w1 = n1;
        }
        pair(w0 & 0xFFFFu);
        pair(w0 >> 16);
        pair(w1 & 0xFFFFu);
        pair(w1 >> 16);
        p += 2;
    }
    if (p < nw) {
        const uint32_t w = p == 0 ? pre.w0 : __ldg(row + (size_t)p * H);
        pair(w & 0xFFFFu);
        pair(w >> 16);
    }
    if (nn & 1u) pair((nw == 0 ? pre.w0 : (nw == 1 ? pre.w1 : __ldg(row + (size_t)nw * H))) & 0xFFFFu);
    if constexpr (KIND == KIND_LJCUT) {
        // rare: a pair within the cut-off band; k_band_stg settles it by the
        // exact FP64 test after this kernel (kept out of this loop so that the
        // loop keeps its registers)
        if (dmin <= 0.0f) {
            const uint32_t k = atomicAdd(c.bandn, 1u);
            if (k < c.n) c.bandq[k] = make_uint2(blockIdx.x, hidx);
        }
    }
}

template <int ND, int KIND, int MODE, int PRM>
__global__ void __launch_bounds__(STG_THREADS, 5) k_force_stg(DevCtx c) {
    extern __shared__ float4 smem_f[];
    __shared__ StgTable T;
    if (blockIdx.x >= c.nblk) {
        if (c.active[blockIdx.x - c.nblk]) stg_nonmembers(c, blockIdx.x - c.nblk, MODE == FM_FORCES_A);
        return;
    }
    const uint4 bd = c.blk[blockIdx.x];
    if (!c.active[bd.x]) return;   // frozen system: forces unchanged
    const SysConst& S = c.sys[bd.x];
    stg_load_table(c, T, blockIdx.x);
    stg_prefetch<ND>(c, T, true);
    const uint32_t cap = c.stg_cap;
    float4* srec = smem_f;
    void* sext = smem_f + cap;
    // the first home atom's global data is requested before the staging
    // wait, so its latency overlaps with the bulk copies
    HomeAtom a0{};
    HomePre p0{};
    const bool has0 = threadIdx.x < T.nhome;
    if (has0) {
        a0 = stg_home<ND, false>(c, T, threadIdx.x);
        p0 = home_pre(c, a0);
    }
    __shared__ uint64_t bar;
    if (!stg_load_bulk<ND, PRM>(c, T, srec, sext, cap, &bar)) return;
    const bool full = T.total <= cap;
    for (uint32_t h = threadIdx.x; h < T.nhome; h += blockDim.x) {
        const HomeAtom a = h == threadIdx.x ? a0 : stg_home<ND, false>(c, T, h);
        const HomePre pre = h == threadIdx.x ? p0 : home_pre(c, a);
        const float4 Qi = pre.Qi;
        Law<KIND> law;
        law.set((KIND == KIND_REPULSION) ? Qi.x * Qi.x : 12.0f * Qi.x * Qi.x, Qi.y, rcp_approx(Qi.y * Qi.y),
                Qi.z);
        float f[3] = {0.f, 0.f, 0.f};
        if (full) force_home<ND, KIND, PRM, true>(c, S, T, srec, sext, cap, a, pre, law, f, h);
        else force_home<ND, KIND, PRM, false>(c, S, T, srec, sext, cap, a, pre, law, f, h);
        c.f32[a.i] = make_float4(f[0], f[1], f[2], 0.f);
        if constexpr (MODE == FM_FORCES_A) {
            using V = typename DVec<ND>::T;
            V av;
            double* ad = reinterpret_cast<double*>(&av);
#pragma unroll
            for (int d = 0; d < (int)(sizeof(V) / 8); d++) ad[d] = 0.0;
            const double m = c.m[a.i];
            if (!(m <= 0.0 || isinf(m))) {
                const float im = c.invm32[a.i];
#pragma unroll
                for (int d = 0; d < ND; d++) ad[d] = (double)(f[d] * im);
            }
            static_cast<V*>(c.a)[a.i] = av;
        }
    }
}

// Settles the home atoms that k_force_stg listed as having a pair within the
// LJ cut-off band: their force is the kernel's FP32 sum plus the exact-test
// corrections, added in list order as if done inline (records are rebuilt
// from global memory, identical to the staged ones).  One CTA of BAND_WARPS
// warps per listed atom: warp w tests the list's chunks w, w + BAND_WARPS,
// ... of 32 entries in parallel (each lane one entry), the corrections are
// collected per entry and one thread adds them in list order.
constexpr uint32_t BAND_WARPS = 3;
constexpr uint32_t BAND_MAXK = 512;   // longer lists: the corrections of one chunk at a time

template <int ND, int KIND, int MODE, int PRM>
__global__ void __launch_bounds__(32 * BAND_WARPS) k_band_stg(DevCtx c) {
    __shared__ StgTable T;
    __shared__ float4 corr[BAND_MAXK];
    __shared__ uint32_t flags[BAND_MAXK / 32];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t nb = min(*c.bandn, c.n);
    for (uint32_t it_k = blockIdx.x; it_k < nb; it_k += gridDim.x) {
        const uint2 it = c.bandq[it_k];
        const uint4 bd = c.blk[it.x];
        const SysConst& S = c.sys[bd.x];
        stg_load_table(c, T, it.x);
        const HomeAtom a = stg_home<ND, false>(c, T, it.y);
        const HomePre pre = home_pre(c, a);
        const float4 Qi = pre.Qi;
        const float4 ri = stg_get<ND>(c, S, T, nullptr, 0u, a.qi);
        const uint32_t wi = stg_wi(ri);
        Law<KIND> law0;
        law0.set(12.0f * Qi.x * Qi.x, Qi.y, rcp_approx(Qi.y * Qi.y), Qi.z);
        // the correction of entry k (FP32 pair force kept or cut wrongly)
        auto entry = [&](uint32_t k, float* cv) -> bool {
            const uint32_t w = __ldg(pre.row + (size_t)(k >> 1) * a.H);
            const uint32_t q = stg_check(c, T, (k & 1u) ? (w >> 16) : (w & 0xFFFFu), a.qi);
            if (q == a.qi) return false;
            const float4 rj = stg_get<ND>(c, S, T, nullptr, 0u, q);
            float r[3];
            stg_disp<ND>(wi, ri, rj, r);
            float d2 = fmaf(r[1], r[1], r[0] * r[0]);
            if constexpr (ND == 3) d2 = fmaf(r[2], r[2], d2);
            Law<KIND> law = law0;
            if constexpr (PRM == 1) {
                const float sg = 0.5f * (Qi.y + c.prm32[stg_global(T, q)].y);
                law.set(law0.e12, sg, rcp_approx(sg * sg), law0.third);
            } else if constexpr (PRM == 2) {
                const float4 Qj = c.prm32[stg_global(T, q)];
                const float sg = 0.5f * (Qi.y + Qj.y);
                law.set(12.0f * Qi.x * Qj.x, sg, rcp_approx(sg * sg), fmaxf(Qi.z, Qj.z));
            }
            float dd;
            const float sc = law.lj_raw(d2, dd);
            if (fabsf(dd) > law.band) return false;
            const bool beyond = lj_beyond_exact_s(c, S, a.i, stg_global(T, q), ND);
            if (beyond == (dd > 0.0f)) return false;   // the FP32 test agreed
            const float sg = beyond ? -sc : sc;
#pragma unroll
            for (int d = 0; d < 3; d++) cv[d] = d < ND ? r[d] * sg : 0.f;
            return true;
        };
        const float4 f0 = c.f32[a.i];
        float f[3] = {f0.x, f0.y, f0.z};
        if (pre.nn <= BAND_MAXK) {
            for (uint32_t t = threadIdx.x; t < BAND_MAXK / 32; t += blockDim.x) flags[t] = 0u;
            __syncthreads();
            for (uint32_t base = 32u * warp; base < pre.nn; base += 32u * BAND_WARPS) {
                const uint32_t k = base + lane;
                float cv[3];
                if (k < pre.nn && entry(k, cv)) {
                    corr[k] = make_float4(cv[0], cv[1], cv[2], 0.f);
                    atomicOr(&flags[k >> 5], 1u << (k & 31u));
                }
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                for (uint32_t wd = 0; wd < (pre.nn + 31u) / 32u; wd++) {
                    uint32_t m = flags[wd];
                    while (m) {
                        const uint32_t k = 32u * wd + (uint32_t)__ffs(m) - 1u;
                        m &= m - 1u;
                        const float4 v = corr[k];
                        f[0] += v.x;
                        f[1] += v.y;
                        f[2] += v.z;
                    }
                }
            }
        } else if (warp == 0) {
            // very long list: one warp, one chunk at a time, in list order
            for (uint32_t base = 0; base < pre.nn; base += 32u) {
                const uint32_t k = base + lane;
                float cv[3] = {0.f, 0.f, 0.f};
                const bool need = k < pre.nn && entry(k, cv);
                uint32_t mask = __ballot_sync(0xFFFFFFFFu, need);
                while (mask) {
                    const int src = __ffs(mask) - 1;
                    mask &= mask - 1u;
#pragma unroll
                    for (int d = 0; d < 3; d++) f[d] += __shfl_sync(0xFFFFFFFFu, cv[d], src);
                }
            }
        }
        if (threadIdx.x == 0) {
            c.f32[a.i] = make_float4(f[0], f[1], f[2], 0.f);
            if constexpr (MODE == FM_FORCES_A) {
                const double m = c.m[a.i];
                if (!(m <= 0.0 || isinf(m))) {
                    const float im = c.invm32[a.i];
                    double* ad = static_cast<double*>(c.a) + (size_t)a.i * (ND == 3 ? 4 : 2);
                    ad[0] = (double)(f[0] * im);
                    ad[1] = (double)(f[1] * im);
                    if constexpr (ND == 3) ad[2] = (double)(f[2] * im);
                }
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// expansion of the staged lists into the row-major global-index lists used by
// the evaluation kernels and the pair listing (same pairs, same order)
// ---------------------------------------------------------------------------
template <int ND>
__global__ void __launch_bounds__(STG_THREADS) k_expand_stg(DevCtx c) {
    __shared__ StgTable T;
    if (blockIdx.x >= c.nblk) return;
    const uint4 bd = c.blk[blockIdx.x];
    const SysConst& S = c.sys[bd.x];
    stg_setup<ND>(c, S, bd, T);
    const uint32_t maxnb = c.maxnb;
    for (uint32_t h = threadIdx.x; h < T.nhome; h += blockDim.x) {
        const HomeAtom a = stg_home<ND>(c, T, h);
        const uint32_t nn = c.nnb[a.i];
        for (uint32_t k = 0; k < nn; k++)
            c.nbr[(size_t)a.i * maxnb + k] = stg_global(T, stg_check(c, T, c.nbr16[stg_entry16(a, maxnb, k)], a.qi));
    }
}

// the inverse: row-major lists (global indices, built on the same cell grid)
// -> staged lists; every neighbour lies in one of the home atom's stencil rows
template <int ND>
__global__ void __launch_bounds__(STG_THREADS) k_compress_stg(DevCtx c) {
    __shared__ StgTable T;
    if (blockIdx.x >= c.nblk) return;
    const uint4 bd = c.blk[blockIdx.x];
    const SysConst& S = c.sys[bd.x];
    stg_setup<ND>(c, S, bd, T);
    const uint32_t maxnb = c.maxnb;
    for (uint32_t h = threadIdx.x; h < T.nhome; h += blockDim.x) {
        const HomeAtom a = stg_home<ND>(c, T, h);
        const uint32_t nn = c.nnb[a.i];
        for (uint32_t k = 0; k < nn; k++) {
            const uint32_t j = c.nbr[(size_t)a.i * maxnb + k];
            uint32_t q = 0xFFFFFFFFu;
            for (uint32_t p = 0; p < T.npiece; p++)
                if (j - T.g0[p] < T.cnt[p]) {
                    q = T.off[p] + (j - T.g0[p]);
                    break;
                }
            if (q > 0xFFFFu) {
                atomicOr(c.status, ST_TILE_OVERFLOW);
                q = a.qi;
            }
            c.nbr16[stg_entry16(a, maxnb, k)] = (uint16_t)q;
        }
    }
    __syncthreads();
    stg_row_nmax<ND>(c, T);
    stg_store_table(c, T, blockIdx.x);
}

// ---------------------------------------------------------------------------
// the list build reads up to 31 records past a row's end: 32 records of padding
size_t stg_smem_build(const DevCtx& c) { return ((size_t)c.stg_cap + 32) * sizeof(float4); }
size_t stg_smem_force(const DevCtx& c) {
    const size_t ext = c.stg_prm == 1 ? sizeof(float) : (c.stg_prm == 2 ? sizeof(float4) : 0);
    return (size_t)c.stg_cap * (sizeof(float4) + ext);
}

template <class K>
static void set_smem(K kern, size_t bytes) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <int ND, int KIND, int MODE>
static void limits_prm(size_t sm) {
    set_smem(k_force_stg<ND, KIND, MODE, 0>, sm);
    set_smem(k_force_stg<ND, KIND, MODE, 1>, sm);
    set_smem(k_force_stg<ND, KIND, MODE, 2>, sm);
}
template <int ND, int KIND>
static void limits_kind(size_t sm) {
    limits_prm<ND, KIND, FM_FORCES>(sm);
    limits_prm<ND, KIND, FM_FORCES_A>(sm);
}
template <int ND>
static void limits_nd(size_t build, size_t force) {
    set_smem(k_build_stg<ND, 0>, build);
    set_smem(k_build_stg<ND, 1>, build);
    limits_kind<ND, KIND_LJCUT>(force);
    limits_kind<ND, KIND_REPULSION>(force);
    limits_kind<ND, KIND_LJREPULSE>(force);
}

// dynamic shared memory limit of every cell-block kernel, raised once to
// the largest stage (4096 atoms of 16 + 16 bytes); called outside stream
// capture.  A limit is an upper bound only: occupancy follows each launch's
// own size.
int stg_set_smem_limits() {
    const size_t most = 4096 * (sizeof(float4) + sizeof(float4));
    limits_nd<3>(most, most);
    limits_nd<2>(most, most);
    return (int)cudaGetLastError();
}

// the tables of every block (after a box change on the same cell grids)
template <int ND>
__global__ void __launch_bounds__(STG_THREADS) k_tables_stg(DevCtx c) {
    __shared__ StgTable T;
    if (blockIdx.x >= c.nblk) return;
    const uint4 bd = c.blk[blockIdx.x];
    stg_setup<ND>(c, c.sys[bd.x], bd, T);
    stg_row_nmax<ND>(c, T);
    stg_store_table(c, T, blockIdx.x);
}

void launch_tables_stg(const DevCtx& c, cudaStream_t s) {
    if (!c.nblk) return;
    if (c.nd == 3) k_tables_stg<3><<<c.nblk, STG_THREADS, 0, s>>>(c);
    else k_tables_stg<2><<<c.nblk, STG_THREADS, 0, s>>>(c);
}

void launch_build_stg(const DevCtx& c, cudaStream_t s) {
    const size_t sm = stg_smem_build(c);
    const unsigned g = c.nblk + c.nsys;
    if (c.nd == 3) {
        if (c.stg_dia) { k_build_stg<3, 1><<<g, STG_THREADS, sm, s>>>(c); }
        else { k_build_stg<3, 0><<<g, STG_THREADS, sm, s>>>(c); }
    } else {
        if (c.stg_dia) { k_build_stg<2, 1><<<g, STG_THREADS, sm, s>>>(c); }
        else { k_build_stg<2, 0><<<g, STG_THREADS, sm, s>>>(c); }
    }
}

constexpr unsigned BAND_CTAS = 2048;

template <int ND, int KIND, int MODE>
static void force_stg_prm(const DevCtx& c, cudaStream_t s) {
    const size_t sm = stg_smem_force(c);
    const unsigned g = c.nblk + c.nsys;
    if (KIND == KIND_LJCUT) cudaMemsetAsync(c.bandn, 0, sizeof(uint32_t), s);
    switch (c.stg_prm) {
        case 0: k_force_stg<ND, KIND, MODE, 0><<<g, STG_THREADS, sm, s>>>(c); break;
        case 1: k_force_stg<ND, KIND, MODE, 1><<<g, STG_THREADS, sm, s>>>(c); break;
        default: k_force_stg<ND, KIND, MODE, 2><<<g, STG_THREADS, sm, s>>>(c); break;
    }
    if (KIND == KIND_LJCUT) {
        switch (c.stg_prm) {
            case 0: k_band_stg<ND, KIND, MODE, 0><<<BAND_CTAS, 32 * BAND_WARPS, 0, s>>>(c); break;
            case 1: k_band_stg<ND, KIND, MODE, 1><<<BAND_CTAS, 32 * BAND_WARPS, 0, s>>>(c); break;
            default: k_band_stg<ND, KIND, MODE, 2><<<BAND_CTAS, 32 * BAND_WARPS, 0, s>>>(c); break;
        }
    }
}

template <int ND, int KIND>
static void force_stg_mode(const DevCtx& c, cudaStream_t s, int mode) {
    if (mode == FM_FORCES_A) force_stg_prm<ND, KIND, FM_FORCES_A>(c, s);
    else force_stg_prm<ND, KIND, FM_FORCES>(c, s);
}

template <int ND>
static void force_stg_kind(const DevCtx& c, cudaStream_t s, int mode) {
    switch (c.kind) {
        case KIND_LJCUT: force_stg_mode<ND, KIND_LJCUT>(c, s, mode); break;
        case KIND_REPULSION: force_stg_mode<ND, KIND_REPULSION>(c, s, mode); break;
        default: force_stg_mode<ND, KIND_LJREPULSE>(c, s, mode); break;
    }
}

void launch_force_stg(const DevCtx& c, cudaStream_t s, int mode) {
    if (c.nd == 3) force_stg_kind<3>(c, s, mode);
    else force_stg_kind<2>(c, s, mode);
}

void launch_expand_stg(const DevCtx& c, cudaStream_t s) {
    if (c.nd == 3) k_expand_stg<3><<<c.nblk, STG_THREADS, 0, s>>>(c);
    else k_expand_stg<2><<<c.nblk, STG_THREADS, 0, s>>>(c);
}

void launch_compress_stg(const DevCtx& c, cudaStream_t s) {
    if (c.nd == 3) k_compress_stg<3><<<c.nblk, STG_THREADS, 0, s>>>(c);
    else k_compress_stg<2><<<c.nblk, STG_THREADS, 0, s>>>(c);
}

}  // namespace parm
