// Per-system "two largest displacements" reduction used by the neighbour-list
// rebuild test (reference: NeighborList::update_list(false), trackers.cpp:23-53).
//
// Each atom contributes its squared FP64 displacement since the last list
// build.  The two largest values per system are kept as the bit patterns of
// non-negative doubles in `top[2s]` (largest) and `top[2s+1]` (second), which
// order like unsigned integers, so atomicMax reproduces the multiset top-2:
// a value that is displaced from the top slot is pushed into the second slot.
// Values are first reduced within a warp (and then a block) when all lanes
// belong to the same system, so a single large system costs two atomics per
// block.
#pragma once
#include "parm_ctx.cuh"

namespace parm {

__device__ __forceinline__ void top2_merge(unsigned long long& a1, unsigned long long& a2,
                                           unsigned long long b1, unsigned long long b2) {
    // merge (a1 >= a2) with (b1 >= b2) into the two largest of the four
    if (b1 > a1) {
        unsigned long long t = a1;
        a1 = b1;
        a2 = (t > b2) ? t : b2;
    } else {
        a2 = (b1 > a2) ? b1 : a2;
    }
}

__device__ __forceinline__ void top2_push(unsigned long long* top, unsigned long long t1,
                                          unsigned long long t2) {
    if (t1 == 0ull) return;
    unsigned long long old = atomicMax(&top[0], t1);
    atomicMax(&top[1], (t1 > old) ? old : t1);
    if (t2) atomicMax(&top[1], t2);
}

// Called by every thread of the block (inactive threads pass valid = false).
// dsq must be >= 0 and finite when valid.
__device__ __forceinline__ void check_accumulate(const DevCtx& c, uint32_t sys_id, bool valid,
                                                 double dsq) {
    __shared__ unsigned long long s1[BLOCK / 32], s2[BLOCK / 32];
    __shared__ uint32_t ssys[BLOCK / 32];
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    // dsq >= 0 (a sum of squares) when valid: its bit pattern orders like its
    // value, and +0 is the pattern 0
    unsigned long long v1 = valid ? (unsigned long long)__double_as_longlong(dsq) : 0ull;
    unsigned long long v2 = 0ull;
    uint32_t sid = valid ? sys_id : 0xFFFFFFFFu;
    // warp-level: lanes that hold no value adopt the warp's first valid system
    unsigned vmask = __ballot_sync(0xFFFFFFFFu, valid);
    uint32_t wsys = 0xFFFFFFFFu;
    if (vmask) wsys = __shfl_sync(0xFFFFFFFFu, sid, __ffs(vmask) - 1);
    bool same = __all_sync(0xFFFFFFFFu, !valid || sid == wsys);
    __syncthreads();
    if (same) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            unsigned long long o1 = __shfl_down_sync(0xFFFFFFFFu, v1, off);
            unsigned long long o2 = __shfl_down_sync(0xFFFFFFFFu, v2, off);
            top2_merge(v1, v2, o1, o2);
        }
        if (lane == 0) {
            s1[warp] = v1;
            s2[warp] = v2;
            ssys[warp] = wsys;
        }
    } else {
        if (valid) top2_push(&c.top[2 * (size_t)sid], v1, 0ull);
        if (lane == 0) {
            s1[warp] = 0ull;
            s2[warp] = 0ull;
            ssys[warp] = 0xFFFFFFFFu;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        // merge runs of warps that share a system, one push per run
        uint32_t cur = 0xFFFFFFFFu;
        unsigned long long a1 = 0ull, a2 = 0ull;
        for (int w = 0; w < BLOCK / 32; w++) {
            if (ssys[w] == 0xFFFFFFFFu) continue;
            if (ssys[w] != cur) {
                if (cur != 0xFFFFFFFFu) top2_push(&c.top[2 * (size_t)cur], a1, a2);
                cur = ssys[w];
                a1 = s1[w];
                a2 = s2[w];
            } else {
                top2_merge(a1, a2, s1[w], s2[w]);
            }
        }
        if (cur != 0xFFFFFFFFu) top2_push(&c.top[2 * (size_t)cur], a1, a2);
    }
}

// squared displacement |x - lastloc|^2 in the reference's order
// ((dx*dx + dy*dy) + dz*dz); FP64 without contraction (callers compile with
// -fmad=false or use this routine, which uses explicit round-to-nearest ops)
template <int ND>
__device__ __forceinline__ double disp_sq(const typename DVec<ND>::T& x, const typename DVec<ND>::T& l);
template <>
__device__ __forceinline__ double disp_sq<3>(const double4& x, const double4& l) {
    double dx = __dsub_rn(x.x, l.x), dy = __dsub_rn(x.y, l.y), dz = __dsub_rn(x.z, l.z);
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}
template <>
__device__ __forceinline__ double disp_sq<2>(const double2& x, const double2& l) {
    double dx = __dsub_rn(x.x, l.x), dy = __dsub_rn(x.y, l.y);
    return __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
}

}  // namespace parm
