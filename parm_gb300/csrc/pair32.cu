// Mixed-precision pair forces: pair displacements, pair laws and per-atom
// force sums in FP32; integration, energy/virial sums and the rebuild test in
// FP64.  Same pair laws as the FP64 path (reference src/interaction.hpp:
// LennardJonesCut 238-281, RepulsionPair 1528-1590, LJRepulsive 119-152).
//
// Displacements come from the coarse/fine split of the FP64 positions
// (posA = trunc(8x)/8 exactly in FP32, posB = the FP32-rounded remainder):
// the coarse difference and its periodic shift are exact in FP32, so the
// displacement is within about one FP32 ulp of the correctly rounded FP64
// value.  With plain FP32 positions relative to cell corners the error is
// about three times larger, which pushes the worst per-atom force error of a
// 10^6-atom LJ liquid above 1e-5 of the rms force.
#include "parm_check.cuh"

namespace parm {

__device__ __forceinline__ bool mobile32(double m) { return !(m <= 0.0 || isinf(m)); }

// FP32 pair law: returns the force scale s (F = r * s) or false beyond cut
template <int KIND>
__device__ __forceinline__ bool scale32(float d2, float eps, float sig, float third, float& s) {
    if constexpr (KIND == KIND_LJCUT || KIND == KIND_LJREPULSE) {
        float isig2 = __frcp_rn(sig * sig);
        float rsq = d2 * isig2;
        float cut2 = (KIND == KIND_LJCUT) ? third * third : 1.0f;
        if (rsq > cut2) return false;
        float ir = __frcp_rn(rsq);
        float ir3 = ir * ir * ir;                   // 1 / rsix
        s = 12.0f * eps * ir3 * (ir3 - 1.0f) * ir * isig2;   // fmagTimesR / dsq
        return true;
    } else {
        float sig2 = sig * sig;
        if (d2 > sig2) return false;
        float R = sqrtf(d2);
        float isig = __frcp_rn(sig);
        float b = 1.0f - R * isig;
        float pw;
        if (third == 2.0f) pw = b;
        else if (third == 2.5f) pw = b * sqrtf(b);
        else pw = powf(b, third - 1.0f);
        s = eps * pw * isig * __frcp_rn(R);
        return true;
    }
}

template <int KIND>
__device__ __forceinline__ float energy32(float d2, float eps, float sig, float third, float m6) {
    if constexpr (KIND == KIND_LJCUT || KIND == KIND_LJREPULSE) {
        float rsq = d2 / (sig * sig);
        float cut2 = (KIND == KIND_LJCUT) ? third * third : 1.0f;
        if (rsq > cut2) return 0.0f;
        float ir3 = 1.0f / (rsq * rsq * rsq);
        float mid = 1.0f - ir3;
        if constexpr (KIND == KIND_LJCUT) return eps * (mid * mid - 1.0f) - eps * (m6 * m6 - 1.0f);
        else return eps * (mid * mid);
    } else {
        if (d2 > sig * sig) return 0.0f;
        float R = sqrtf(d2);
        float b = 1.0f - R / sig;
        float pw = (third == 2.0f) ? b * b : powf(b, third);
        return eps * pw / third;
    }
}

template <int ND>
__device__ __forceinline__ void disp3(const SysConst& S, const float4& Ai, const float4& Bi,
                                      const float4& Aj, const float4& Bj, float* r) {
    r[0] = disp32(Ai.x, Aj.x, Bi.x, Bj.x, S.Lhi[0], S.Llo[0], S.invLf[0]);
    r[1] = disp32(Ai.y, Aj.y, Bi.y, Bj.y, S.Lhi[1], S.Llo[1], S.invLf[1]);
    r[2] = 0.0f;
    if constexpr (ND == 3) r[2] = disp32(Ai.z, Aj.z, Bi.z, Bj.z, S.Lhi[2], S.Llo[2], S.invLf[2]);
}

template <int ND, int KIND, int MODE>
__global__ void __launch_bounds__(BLOCK) k_force32(DevCtx c) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = i < c.n;
    const uint32_t uni = c.uniform;
    float f[3] = {0.f, 0.f, 0.f};
    uint32_t s = 0;
    bool member = false;
    if (active) {
        s = c.atom_sys[i];
        member = c.rank[i] != NOT_MEMBER;
    }
    if (member) {
        const SysConst& S = c.sys[s];
        const float4 Ai = c.posA[i], Bi = c.posB[i];
        const float4 Qi = c.prm32[i];   // (sqrt(eps), sigma, third, m6)
        const bool need_j = (uni & (UNI_EPS | UNI_SIG | UNI_THIRD)) != (UNI_EPS | UNI_SIG | UNI_THIRD);
        const uint32_t nn = c.nnb[i];
        const uint32_t* nb = c.nbr + i;
        for (uint32_t k = 0; k < nn; k++) {
            const uint32_t j = __ldg(nb + (size_t)k * c.nalloc);
            const float4 Aj = c.posA[j], Bj = c.posB[j];
            float r[3];
            disp3<ND>(S, Ai, Bi, Aj, Bj, r);
            float d2 = r[0] * r[0] + r[1] * r[1];
            if constexpr (ND == 3) d2 += r[2] * r[2];
            float eps = Qi.x * Qi.x, sig = Qi.y, third = Qi.z;
            if (need_j) {
                const float4 Qj = c.prm32[j];
                eps = Qi.x * Qj.x;
                sig = 0.5f * (Qi.y + Qj.y);
                third = (KIND == KIND_LJCUT) ? fmaxf(Qi.z, Qj.z) : 0.5f * (Qi.z + Qj.z);
            }
            float sc;
            if (!scale32<KIND>(d2, eps, sig, third, sc)) continue;
#pragma unroll
            for (int d = 0; d < ND; d++) f[d] += r[d] * sc;
        }
    }
    if (active) {
        c.f32[i] = make_float4(f[0], f[1], f[2], 0.f);
        using V = typename DVec<ND>::T;
        if constexpr (MODE != FM_FORCES) {
            const StepParams& P = *c.params;
            const double m = c.m[i];
            const float im = c.invm32[i];
            V av;
            double* a = reinterpret_cast<double*>(&av);
#pragma unroll
            for (int d = 0; d < (int)(sizeof(V) / 8); d++) a[d] = 0.0;
            bool mob = (MODE == FM_SOL) ? !(m == 0.0 || isinf(m)) : mobile32(m);
            if (mob) {
                const float imm = (MODE == FM_SOL && !mobile32(m)) ? (float)(1.0 / m) : im;
#pragma unroll
                for (int d = 0; d < ND; d++) a[d] = (double)(f[d] * imm);
            }
            static_cast<V*>(c.a)[i] = av;
            if constexpr (MODE == FM_VERLET || MODE == FM_DAMPED || MODE == FM_SOL) {
                V vv = static_cast<const V*>(c.v)[i];
                double* v = reinterpret_cast<double*>(&vv);
                const double h = (MODE == FM_VERLET) ? P.dt_half : P.dtc2;
                if (mob) {
#pragma unroll
                    for (int d = 0; d < ND; d++) v[d] = v[d] + a[d] * h;
                    static_cast<V*>(c.v)[i] = vv;
                } else if (MODE == FM_SOL) {
#pragma unroll
                    for (int d = 0; d < ND; d++) v[d] = 0.0;
                    static_cast<V*>(c.v)[i] = vv;
                }
            }
        }
    }
    if constexpr (MODE == FM_VERLET || MODE == FM_DAMPED || MODE == FM_SOL) {
        double dsq = 0.0;
        bool valid = false;
        if (member) {
            dsq = disp_sq<ND>(static_cast<const typename DVec<ND>::T*>(c.x)[i],
                              static_cast<const typename DVec<ND>::T*>(c.lastloc)[i]);
            valid = !(dsq != dsq);
        }
        check_accumulate(c, s, valid, dsq);
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
        const float4 Ai = c.posA[i], Bi = c.posB[i];
        const float4 Qi = c.prm32[i];
        const uint32_t nn = c.nnb[i];
        for (uint32_t k = 0; k < nn; k++) {
            const uint32_t j = c.nbr[(size_t)k * c.nalloc + i];
            if (c.rank[j] > ri) continue;
            float r[3];
            disp3<ND>(S, Ai, Bi, c.posA[j], c.posB[j], r);
            float d2 = r[0] * r[0] + r[1] * r[1];
            if constexpr (ND == 3) d2 += r[2] * r[2];
            const float4 Qj = c.prm32[j];
            float eps = Qi.x * Qj.x, sig = 0.5f * (Qi.y + Qj.y);
            float third = (KIND == KIND_LJCUT) ? fmaxf(Qi.z, Qj.z) : 0.5f * (Qi.z + Qj.z);
            float m6 = (KIND == KIND_LJCUT) ? (Qj.z > Qi.z ? Qj.w : Qi.w) : 0.f;
            if (what == EV_ENERGY || what == EV_CONTACTS || what == EV_OVERLAPS) {
                float e = energy32<KIND>(d2, eps, sig, third, m6);
                if (what == EV_ENERGY) acc[0] += (double)e;
                else if (what == EV_CONTACTS) acc[0] += (e != 0.0f) ? 1.0 : 0.0;
                else acc[0] += (e > 0.0f) ? 1.0 : 0.0;
            } else {
                float sc = 0.f;
                float fo[3] = {0.f, 0.f, 0.f};
                if (scale32<KIND>(d2, eps, sig, third, sc)) {
#pragma unroll
                    for (int d = 0; d < ND; d++) fo[d] = r[d] * sc;
                }
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

template <int ND, int KIND>
static void force32_nd_kind(const DevCtx& c, cudaStream_t s, int mode) {
    unsigned g = grid_for(c.n);
    switch (mode) {
        case FM_FORCES: k_force32<ND, KIND, FM_FORCES><<<g, BLOCK, 0, s>>>(c); break;
        case FM_FORCES_A: k_force32<ND, KIND, FM_FORCES_A><<<g, BLOCK, 0, s>>>(c); break;
        case FM_VERLET: k_force32<ND, KIND, FM_VERLET><<<g, BLOCK, 0, s>>>(c); break;
        case FM_DAMPED: k_force32<ND, KIND, FM_DAMPED><<<g, BLOCK, 0, s>>>(c); break;
        default: k_force32<ND, KIND, FM_SOL><<<g, BLOCK, 0, s>>>(c); break;
    }
}

template <int ND>
static void force32_nd(const DevCtx& c, cudaStream_t s, int mode) {
    if (c.kind == KIND_LJCUT) force32_nd_kind<ND, KIND_LJCUT>(c, s, mode);
    else if (c.kind == KIND_REPULSION) force32_nd_kind<ND, KIND_REPULSION>(c, s, mode);
    else force32_nd_kind<ND, KIND_LJREPULSE>(c, s, mode);
}

void launch_force32(const DevCtx& c, cudaStream_t s, int mode) {
    if (c.nd == 3) force32_nd<3>(c, s, mode); else force32_nd<2>(c, s, mode);
}

template <int ND>
static void eval32_nd(const DevCtx& c, cudaStream_t s, int what) {
    unsigned g = grid_for(c.n);
    if (c.kind == KIND_LJCUT) k_eval32<ND, KIND_LJCUT><<<g, BLOCK, 0, s>>>(c, what);
    else if (c.kind == KIND_REPULSION) k_eval32<ND, KIND_REPULSION><<<g, BLOCK, 0, s>>>(c, what);
    else k_eval32<ND, KIND_LJREPULSE><<<g, BLOCK, 0, s>>>(c, what);
}

void launch_eval32(const DevCtx& c, cudaStream_t s, int what) {
    if (c.nd == 3) eval32_nd<3>(c, s, what); else eval32_nd<2>(c, s, what);
}

}  // namespace parm
