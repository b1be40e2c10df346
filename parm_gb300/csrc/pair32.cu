// Mixed-precision pair forces: pair displacements, pair laws and per-atom
// force sums in FP32; integration, energy/virial sums and the rebuild test in
// FP64.  Same pair laws as the FP64 path (reference src/interaction.hpp:
// LennardJonesCut 238-281, RepulsionPair 1528-1590, LJRepulsive 119-152).
//
// Displacements come from the coarse/fine split of the FP64 positions
// (pos[2i] = trunc(8x)/8 exactly in FP32, pos[2i+1] = the FP32-rounded remainder):
// the coarse difference and its periodic shift are exact in FP32, so the
// displacement is within about one FP32 ulp of the correctly rounded FP64
// value.  With plain FP32 positions relative to cell corners the error is
// about three times larger, which pushes the worst per-atom force error of a
// 10^6-atom LJ liquid above 1e-5 of the rms force.
#include <algorithm>

#include "parm_check.cuh"
#include "parm_pair32.cuh"

namespace parm {

__device__ __forceinline__ bool mobile32(double m) { return !(m <= 0.0 || isinf(m)); }

__device__ __noinline__ bool lj_beyond_exact(const DevCtx& c, const SysConst& S, uint32_t i, uint32_t j,
                                             int nd) {
    const double* xi = reinterpret_cast<const double*>(c.x) + (size_t)i * (nd == 3 ? 4 : 2);
    const double* xj = reinterpret_cast<const double*>(c.x) + (size_t)j * (nd == 3 ? 4 : 2);
    double dsq = 0.0;
    double sq[3] = {0.0, 0.0, 0.0};
    for (int d = 0; d < nd; d++) {
        double r = remainder_exact(__dsub_rn(xi[d], xj[d]), S.L[d], S.invL[d], S.halfL[d]);
        sq[d] = __dmul_rn(r, r);
    }
    dsq = __dadd_rn(sq[0], sq[1]);
    if (nd == 3) dsq = __dadd_rn(dsq, sq[2]);
    const AtomPrm A = c.prm[i], B = c.prm[j];
    double sig = __dmul_rn(__dadd_rn(A.p1, B.p1), 0.5);
    double cut = B.p2 > A.p2 ? B.p2 : A.p2;
    double rsq = __ddiv_rn(dsq, __dmul_rn(sig, sig));
    return rsq > __dmul_rn(cut, cut);
}

template <int ND>
__device__ __forceinline__ void disp3(const SysConst& S, const float4& Ai, const float4& Bi,
                                      const float4& Aj, const float4& Bj, float* r) {
    r[0] = disp32(Ai.x, Aj.x, Bi.x, Bj.x, S.Lhi[0], S.Llo[0], S.invLf[0]);
    r[1] = disp32(Ai.y, Aj.y, Bi.y, Bj.y, S.Lhi[1], S.Llo[1], S.invLf[1]);
    r[2] = 0.0f;
    if constexpr (ND == 3) r[2] = disp32(Ai.z, Aj.z, Bi.z, Bj.z, S.Lhi[2], S.Llo[2], S.invLf[2]);
}

// TPA threads share one atom: lane `sub` of the group takes neighbours
// sub, sub + TPA, ...; the partial forces are summed with shuffles.  The lists
// are row-major and in cell order, so the TPA lanes of a group read one
// contiguous stretch of the list and gather neighbours that mostly share
// cache lines (an L1 line per lane per pair when each lane works on a
// different atom).
template <int ND, int KIND, int MODE, int TPA, int UNR>
__global__ void __launch_bounds__(BLOCK) k_force32(DevCtx c) {
    const uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t i = gt / TPA;
    const uint32_t sub = gt % TPA;
    const bool active = i < c.n && c.active[c.atom_sys[i]];
    const uint32_t uni = c.uniform;
    float f[3] = {0.f, 0.f, 0.f};
    bool member = false;
    uint32_t s = 0;
    if (active) {
        s = c.atom_sys[i];
        member = c.rank[i] != NOT_MEMBER;
    }
    if (member) {
        const SysConst& S = c.sys[s];
        float4 Ai, Bi;
        ld_pos(c.pos, i, Ai, Bi);
        const float4 Qi = c.prm32[i];   // (sqrt(eps), sigma, third, m6)
        const bool need_j = (uni & (UNI_EPS | UNI_SIG | UNI_THIRD)) != (UNI_EPS | UNI_SIG | UNI_THIRD);
        const float e_u = (KIND == KIND_REPULSION) ? Qi.x * Qi.x : 12.0f * Qi.x * Qi.x;
        const float is_u = __fdividef(1.0f, Qi.y * Qi.y);
        const uint32_t nn = c.nnb[i];
        const uint32_t* nb = c.nbr + (size_t)i * c.maxnb;
        bool any_band = false;
        // UNR neighbours per lane and iteration: one vector index load (rows are
        // padded to a multiple of 8 entries) and UNR gathers in flight
#pragma unroll 1
        for (uint32_t k = UNR * sub; k < nn; k += UNR * TPA) {
            uint32_t js[4];
            if constexpr (UNR == 4) {
                const uint4 jj = __ldg(reinterpret_cast<const uint4*>(nb + k));
                js[0] = jj.x; js[1] = jj.y; js[2] = jj.z; js[3] = jj.w;
            } else if constexpr (UNR == 2) {
                const uint2 jj = __ldg(reinterpret_cast<const uint2*>(nb + k));
                js[0] = jj.x; js[1] = jj.y;
            } else {
                js[0] = __ldg(nb + k);
            }
            float4 Aj[UNR], Bj[UNR];
#pragma unroll
            for (int u = 0; u < UNR; u++) {
                if (k + u < nn) ld_pos(c.pos, js[u], Aj[u], Bj[u]);
                else Aj[u] = Bj[u] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
#pragma unroll
            for (int u = 0; u < UNR; u++) {
                if (k + u >= nn) break;
                const uint32_t j = js[u];
                float r[3];
                disp3<ND>(S, Ai, Bi, Aj[u], Bj[u], r);
                float d2 = r[0] * r[0] + r[1] * r[1];
                if constexpr (ND == 3) d2 += r[2] * r[2];
                float e12 = e_u, sig = Qi.y, isig2 = is_u, third = Qi.z;
                if (need_j) {
                    const float4 Qj = __ldg(&c.prm32[j]);
                    const float eps = Qi.x * Qj.x;
                    e12 = (KIND == KIND_REPULSION) ? eps : 12.0f * eps;
                    sig = 0.5f * (Qi.y + Qj.y);
                    isig2 = __fdividef(1.0f, sig * sig);
                    third = cut_kind<KIND>() ? fmaxf(Qi.z, Qj.z) : 0.5f * (Qi.z + Qj.z);
                }
                bool near_cut;
                float sc = scale32<KIND>(d2, e12, sig, isig2, third, near_cut);
                if constexpr (cut_kind<KIND>()) {
                    // pairs within the band are added here as if inside the
                    // cut-off and settled by the exact test after the loop
                    if (near_cut) {
                        const float rsq = d2 * isig2;
                        const float ir = __fdividef(1.0f, rsq);
                        const float ir3 = ir * ir * ir;
                        sc = e12 * ir3 * (ir3 - 1.0f) * ir * isig2;
                        any_band = true;
                    }
                }
#pragma unroll
                for (int d = 0; d < ND; d++) f[d] = fmaf(r[d], sc, f[d]);
            }
        }
        if constexpr (cut_kind<KIND>()) {
            if (any_band) {
                // rare: remove the band pairs that the exact FP64 test puts
                // beyond the cut-off (same FP32 contribution as added above)
                for (uint32_t k0 = UNR * sub; k0 < nn; k0 += UNR * TPA)
                for (uint32_t k = k0; k < k0 + UNR && k < nn; k++) {
                    const uint32_t j = nb[k];
                    float4 Aj, Bj;
                    ld_pos(c.pos, j, Aj, Bj);
                    float r[3];
                    disp3<ND>(S, Ai, Bi, Aj, Bj, r);
                    float d2 = r[0] * r[0] + r[1] * r[1];
                    if constexpr (ND == 3) d2 += r[2] * r[2];
                    float e12 = e_u, sig = Qi.y, isig2 = is_u, third = Qi.z;
                    if (need_j) {
                        const float4 Qj = c.prm32[j];
                        e12 = 12.0f * Qi.x * Qj.x;
                        sig = 0.5f * (Qi.y + Qj.y);
                        isig2 = __fdividef(1.0f, sig * sig);
                        third = fmaxf(Qi.z, Qj.z);
                    }
                    const float rsq = d2 * isig2;
                    const float cut2 = third * third;
                    if (fabsf(rsq - cut2) > CUT_BAND * cut2) continue;
                    if (!lj_beyond_exact(c, S, i, j, ND)) continue;
                    const float ir = __fdividef(1.0f, rsq);
                    const float ir3 = ir * ir * ir;
                    const float sc = e12 * ir3 * (ir3 - 1.0f) * ir * isig2;
#pragma unroll
                    for (int d = 0; d < ND; d++) f[d] = fmaf(-r[d], sc, f[d]);
                }
            }
        }
    }
    if constexpr (TPA > 1) {
#pragma unroll
        for (int o = TPA / 2; o > 0; o >>= 1) {
#pragma unroll
            for (int d = 0; d < 3; d++) f[d] += __shfl_xor_sync(0xFFFFFFFFu, f[d], o);
        }
    }
    if (active && sub == 0) {
        c.f32[i] = make_float4(f[0], f[1], f[2], 0.f);
        if constexpr (MODE == FM_FORCES_A) {
            // Collection::set_forces(true): a = f/m, zero for m <= 0 or inf
            using V = typename DVec<ND>::T;
            V av;
            double* a = reinterpret_cast<double*>(&av);
#pragma unroll
            for (int d = 0; d < (int)(sizeof(V) / 8); d++) a[d] = 0.0;
            if (mobile32(c.m[i])) {
                const float im = c.invm32[i];
#pragma unroll
                for (int d = 0; d < ND; d++) a[d] = (double)(f[d] * im);
            }
            static_cast<V*>(c.a)[i] = av;
        }
    }
}

// Tiled variant: one CTA per tile of TILE_ATOMS atoms, TPA threads per atom.
// The tile's entries (distinct neighbour images) are staged once in shared
// memory in the tile frame: coarse part R = X_j - A0 + img * Lhi (exact in
// FP32) and fine part F = xf_j + img * Llo; every pair then reads its
// neighbour from shared memory through a 16-bit entry number and the
// displacement is (R_i - R_j) + (F_i - F_j), with no per-pair minimum image.
template <int ND, int KIND, int MODE, int TPA>
__global__ void __launch_bounds__(TILE_ATOMS * TPA) k_force32t(DevCtx c) {
    extern __shared__ float4 tile_smem[];
    float4* sR = tile_smem;
    float4* sF = tile_smem + TILE_ECAP;
    const uint32_t t = blockIdx.x;
    const uint32_t tid = threadIdx.x;
    const uint32_t s = c.tile_sys[t];
    if (!c.active[s]) return;   // frozen system: forces unchanged
    const SysConst& S = c.sys[s];
    const uint32_t ne = c.tile_ne[t];
    const float4 A0 = c.tile_anchor[t];
    const unsigned long long* ent = c.tile_ent + (size_t)t * TILE_ECAP;
    for (uint32_t e = tid; e < ne; e += blockDim.x) {
        const unsigned long long key = ent[e];
        const uint32_t j = (uint32_t)(key >> 24);
        const float i0 = (float)((int)(key & 255u) - 128);
        const float i1 = (float)((int)((key >> 8) & 255u) - 128);
        const float i2 = (float)((int)((key >> 16) & 255u) - 128);
        float4 Aj, Bj;
        ld_pos(c.pos, j, Aj, Bj);
        sR[e] = make_float4(__fmaf_rn(i0, S.Lhi[0], Aj.x - A0.x), __fmaf_rn(i1, S.Lhi[1], Aj.y - A0.y),
                            ND == 3 ? __fmaf_rn(i2, S.Lhi[2], Aj.z - A0.z) : 0.f, 0.f);
        sF[e] = make_float4(__fmaf_rn(i0, S.Llo[0], Bj.x), __fmaf_rn(i1, S.Llo[1], Bj.y),
                            ND == 3 ? __fmaf_rn(i2, S.Llo[2], Bj.z) : 0.f, 0.f);
    }
    __syncthreads();
    const uint32_t a = tid / TPA, sub = tid % TPA;
    const uint32_t i = c.tile_atom0[t] + a;
    const bool active = a < c.tile_natom[t];
    const uint32_t uni = c.uniform;
    float f[3] = {0.f, 0.f, 0.f};
    if (active && c.rank[i] != NOT_MEMBER) {
        float4 Ai, Bi;
        ld_pos(c.pos, i, Ai, Bi);
        const uint32_t mc = c.atom_img[i];
        const float m0 = (float)((int)(mc & 255u) - 128), m1 = (float)((int)((mc >> 8) & 255u) - 128);
        const float m2 = (float)((int)((mc >> 16) & 255u) - 128);
        const float R0 = __fmaf_rn(-m0, S.Lhi[0], Ai.x - A0.x), F0 = __fmaf_rn(-m0, S.Llo[0], Bi.x);
        const float R1 = __fmaf_rn(-m1, S.Lhi[1], Ai.y - A0.y), F1 = __fmaf_rn(-m1, S.Llo[1], Bi.y);
        const float R2 = ND == 3 ? __fmaf_rn(-m2, S.Lhi[2], Ai.z - A0.z) : 0.f;
        const float F2 = ND == 3 ? __fmaf_rn(-m2, S.Llo[2], Bi.z) : 0.f;
        const float4 Qi = c.prm32[i];
        const bool need_j = (uni & (UNI_EPS | UNI_SIG | UNI_THIRD)) != (UNI_EPS | UNI_SIG | UNI_THIRD);
        const float e_u = (KIND == KIND_REPULSION) ? Qi.x * Qi.x : 12.0f * Qi.x * Qi.x;
        const float is_u = __fdividef(1.0f, Qi.y * Qi.y);
        const uint32_t nn = c.nnb[i];
        const uint16_t* lst = c.tile_lst + (size_t)t * c.maxnb * TILE_ATOMS + a;
        bool any_band = false;
#pragma unroll 2
        for (uint32_t k = sub; k < nn; k += TPA) {
            const uint32_t e = lst[(size_t)k * TILE_ATOMS];
            const float4 R = sR[e], F = sF[e];
            float r[3];
            r[0] = (R0 - R.x) + (F0 - F.x);
            r[1] = (R1 - R.y) + (F1 - F.y);
            r[2] = (R2 - R.z) + (F2 - F.z);
            float d2 = r[0] * r[0] + r[1] * r[1];
            if constexpr (ND == 3) d2 += r[2] * r[2];
            float e12 = e_u, sig = Qi.y, isig2 = is_u, third = Qi.z;
            if (need_j) {
                const uint32_t j = (uint32_t)(c.tile_ent[(size_t)t * TILE_ECAP + e] >> 24);
                const float4 Qj = __ldg(&c.prm32[j]);
                const float eps = Qi.x * Qj.x;
                e12 = (KIND == KIND_REPULSION) ? eps : 12.0f * eps;
                sig = 0.5f * (Qi.y + Qj.y);
                isig2 = __fdividef(1.0f, sig * sig);
                third = cut_kind<KIND>() ? fmaxf(Qi.z, Qj.z) : 0.5f * (Qi.z + Qj.z);
            }
            bool near_cut;
            float sc = scale32<KIND>(d2, e12, sig, isig2, third, near_cut);
            if constexpr (cut_kind<KIND>()) {
                if (near_cut) {   // settled by the exact test after the loop
                    const float rsq = d2 * isig2;
                    const float ir = __fdividef(1.0f, rsq);
                    const float ir3 = ir * ir * ir;
                    sc = e12 * ir3 * (ir3 - 1.0f) * ir * isig2;
                    any_band = true;
                }
            }
#pragma unroll
            for (int d = 0; d < ND; d++) f[d] = fmaf(r[d], sc, f[d]);
        }
        if constexpr (cut_kind<KIND>()) {
            if (any_band) {
                for (uint32_t k = sub; k < nn; k += TPA) {
                    const uint32_t e = lst[(size_t)k * TILE_ATOMS];
                    const float4 R = sR[e], F = sF[e];
                    float r[3];
                    r[0] = (R0 - R.x) + (F0 - F.x);
                    r[1] = (R1 - R.y) + (F1 - F.y);
                    r[2] = (R2 - R.z) + (F2 - F.z);
                    float d2 = r[0] * r[0] + r[1] * r[1];
                    if constexpr (ND == 3) d2 += r[2] * r[2];
                    const uint32_t j = (uint32_t)(c.tile_ent[(size_t)t * TILE_ECAP + e] >> 24);
                    float e12 = e_u, isig2 = is_u, third = Qi.z;
                    if (need_j) {
                        const float4 Qj = c.prm32[j];
                        e12 = 12.0f * Qi.x * Qj.x;
                        const float sig = 0.5f * (Qi.y + Qj.y);
                        isig2 = __fdividef(1.0f, sig * sig);
                        third = fmaxf(Qi.z, Qj.z);
                    }
                    const float rsq = d2 * isig2;
                    const float cut2 = third * third;
                    if (fabsf(rsq - cut2) > CUT_BAND * cut2) continue;
                    if (!lj_beyond_exact(c, S, i, j, ND)) continue;
                    const float ir = __fdividef(1.0f, rsq);
                    const float ir3 = ir * ir * ir;
                    const float sc = e12 * ir3 * (ir3 - 1.0f) * ir * isig2;
#pragma unroll
                    for (int d = 0; d < ND; d++) f[d] = fmaf(-r[d], sc, f[d]);
                }
            }
        }
    }
    if constexpr (TPA > 1) {
#pragma unroll
        for (int o = TPA / 2; o > 0; o >>= 1) {
#pragma unroll
            for (int d = 0; d < 3; d++) f[d] += __shfl_xor_sync(0xFFFFFFFFu, f[d], o);
        }
    }
    if (active && sub == 0) {
        c.f32[i] = make_float4(f[0], f[1], f[2], 0.f);
        if constexpr (MODE == FM_FORCES_A) {
            using V = typename DVec<ND>::T;
            V av;
            double* ap = reinterpret_cast<double*>(&av);
#pragma unroll
            for (int d = 0; d < (int)(sizeof(V) / 8); d++) ap[d] = 0.0;
            if (mobile32(c.m[i])) {
                const float im = c.invm32[i];
#pragma unroll
                for (int d = 0; d < ND; d++) ap[d] = (double)(f[d] * im);
            }
            static_cast<V*>(c.a)[i] = av;
        }
    }
}

template <int ND, int KIND>
__global__ void __launch_bounds__(BLOCK) k_eval32(DevCtx c, int what) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const int ncomp = (what == EV_STRESS) ? ND * ND : 1;
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const uint32_t ri = c.rank[i];
    if (ri != NOT_MEMBER) {
        const SysConst& S = c.sys[c.atom_sys[i]];
        const float4 Ai = c.pos[2 * (size_t)(i)], Bi = c.pos[2 * (size_t)(i) + 1];
        const float4 Qi = c.prm32[i];
        const uint32_t nn = c.nnb[i];
        for (uint32_t k = 0; k < nn; k++) {
            const uint32_t j = c.nbr[(size_t)i * c.maxnb + k];
            if (c.rank[j] > ri) continue;
            float r[3];
            disp3<ND>(S, Ai, Bi, c.pos[2 * (size_t)(j)], c.pos[2 * (size_t)(j) + 1], r);
            float d2 = r[0] * r[0] + r[1] * r[1];
            if constexpr (ND == 3) d2 += r[2] * r[2];
            const float4 Qj = c.prm32[j];
            float eps = Qi.x * Qj.x, sig = 0.5f * (Qi.y + Qj.y);
            float third = cut_kind<KIND>() ? fmaxf(Qi.z, Qj.z) : 0.5f * (Qi.z + Qj.z);
            float m6 = cut_kind<KIND>() ? (Qj.z > Qi.z ? Qj.w : Qi.w) : 0.f;
            if (what == EV_ENERGY || what == EV_CONTACTS || what == EV_OVERLAPS) {
                float e = energy32<KIND>(d2, eps, sig, third, m6);
                if (what == EV_ENERGY) acc[0] += (double)e;
                else if (what == EV_CONTACTS) acc[0] += (e != 0.0f) ? 1.0 : 0.0;
                else acc[0] += (e > 0.0f) ? 1.0 : 0.0;
            } else {
                bool near_cut;
                const float e12 = (KIND == KIND_REPULSION) ? eps : 12.0f * eps;
                float sc = scale32<KIND>(d2, e12, sig, 1.0f / (sig * sig), third, near_cut);
                if constexpr (cut_kind<KIND>()) {
                    if (near_cut && lj_beyond_exact(c, S, i, j, ND)) sc = 0.0f;
                    else if (near_cut) {
                        const float rsq = d2 / (sig * sig);
                        const float ir3 = 1.0f / (rsq * rsq * rsq);
                        sc = e12 * ir3 * (ir3 - 1.0f) / d2;
                    }
                }
                float fo[3] = {0.f, 0.f, 0.f};
#pragma unroll
                for (int d = 0; d < ND; d++) fo[d] = r[d] * sc;
                if (what == EV_VIRIAL) {
                    double p = 0.0;
#pragma unroll
                    for (int d = 0; d < ND; d++) p += (double)r[d] * (double)fo[d];
                    acc[0] += p;
                } else {
#pragma unroll
                    for (int aa = 0; aa < ND; aa++)
#pragma unroll
                        for (int bb = 0; bb < ND; bb++) acc[aa * ND + bb] += (double)r[aa] * (double)fo[bb];
                }
            }
        }
    }
    for (int q = 0; q < ncomp; q++) c.red[(size_t)q * c.n + i] = acc[q];
}

// launch configuration: c.tpa = threads per atom, c.unr = neighbours per lane
// and iteration
template <int ND, int KIND, int MODE, int UNR>
static void force32_unr(const DevCtx& c, cudaStream_t s) {
    const uint32_t t = c.tpa;
    const unsigned g = grid_for((uint32_t)std::min<uint64_t>((uint64_t)c.n * t, 0xFFFFFFFFull));
    switch (t) {
        case 32: k_force32<ND, KIND, MODE, 32, UNR><<<g, BLOCK, 0, s>>>(c); break;
        case 16: k_force32<ND, KIND, MODE, 16, UNR><<<g, BLOCK, 0, s>>>(c); break;
        case 8: k_force32<ND, KIND, MODE, 8, UNR><<<g, BLOCK, 0, s>>>(c); break;
        case 4: k_force32<ND, KIND, MODE, 4, UNR><<<g, BLOCK, 0, s>>>(c); break;
        default: k_force32<ND, KIND, MODE, 1, UNR><<<grid_for(c.n), BLOCK, 0, s>>>(c); break;
    }
}

template <int ND, int KIND, int MODE>
static void force32_tpa(const DevCtx& c, cudaStream_t s) {
    if (c.tiled && c.ntile) {
        const size_t smem = 2 * (size_t)TILE_ECAP * sizeof(float4);
        switch (c.tpa) {
            case 4: k_force32t<ND, KIND, MODE, 4><<<c.ntile, TILE_ATOMS * 4, smem, s>>>(c); break;
            case 2: k_force32t<ND, KIND, MODE, 2><<<c.ntile, TILE_ATOMS * 2, smem, s>>>(c); break;
            default: k_force32t<ND, KIND, MODE, 1><<<c.ntile, TILE_ATOMS, smem, s>>>(c); break;
        }
        return;
    }
    if (c.unr == 4) force32_unr<ND, KIND, MODE, 4>(c, s);
    else if (c.unr == 2) force32_unr<ND, KIND, MODE, 2>(c, s);
    else force32_unr<ND, KIND, MODE, 1>(c, s);
}

template <int ND, int KIND>
static void force32_nd_kind(const DevCtx& c, cudaStream_t s, int mode) {
    if (mode == FM_FORCES_A) force32_tpa<ND, KIND, FM_FORCES_A>(c, s);
    else force32_tpa<ND, KIND, FM_FORCES>(c, s);
}

template <int ND>
static void force32_nd(const DevCtx& c, cudaStream_t s, int mode) {
    if (c.kind == KIND_LJCUT) force32_nd_kind<ND, KIND_LJCUT>(c, s, mode);
    else if (c.kind == KIND_LJATTRACT) force32_nd_kind<ND, KIND_LJATTRACT>(c, s, mode);
    else if (c.kind == KIND_REPULSION) force32_nd_kind<ND, KIND_REPULSION>(c, s, mode);
    else force32_nd_kind<ND, KIND_LJREPULSE>(c, s, mode);
}

void launch_force32(const DevCtx& c, cudaStream_t s, int mode) {
    if (c.staged) launch_force_stg(c, s, mode);
    else if (c.nd == 3) force32_nd<3>(c, s, mode);
    else force32_nd<2>(c, s, mode);
}

template <int ND>
static void eval32_nd(const DevCtx& c, cudaStream_t s, int what) {
    unsigned g = grid_for(c.n);
    if (c.kind == KIND_LJCUT) k_eval32<ND, KIND_LJCUT><<<g, BLOCK, 0, s>>>(c, what);
    else if (c.kind == KIND_LJATTRACT) k_eval32<ND, KIND_LJATTRACT><<<g, BLOCK, 0, s>>>(c, what);
    else if (c.kind == KIND_REPULSION) k_eval32<ND, KIND_REPULSION><<<g, BLOCK, 0, s>>>(c, what);
    else k_eval32<ND, KIND_LJREPULSE><<<g, BLOCK, 0, s>>>(c, what);
}

void launch_eval32(const DevCtx& c, cudaStream_t s, int what) {
    if (c.nd == 3) eval32_nd<3>(c, s, what); else eval32_nd<2>(c, s, what);
}

}  // namespace parm
