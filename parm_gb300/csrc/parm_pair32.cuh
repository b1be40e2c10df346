// FP32 pair laws shared by the mixed-precision pair kernels (pair32.cu,
// staged.cu).  Same laws as the FP64 path (reference src/interaction.hpp:
// LennardJonesCut 238-281, RepulsionPair 1528-1590, LJRepulsive 119-152,
// LJAttractCut 154-236).
#pragma once
#include "parm_ctx.cuh"

namespace parm {

// The reference's truncated LJ force jumps by ~0.044 eps/sigma at the cut-off
// (LennardJonesCut::forces, src/interaction.hpp:263-271: zero for
// rsq > cut^2).  A pair whose FP32 rsq lies within 4e-6 (relative) of cut^2 is
// therefore classified with the exact FP64 test of the reference, so the set
// of interacting pairs is identical to the FP64 path's.  (RepulsionPair and
// LJRepulsive forces vanish continuously at their cut-offs.)
constexpr float CUT_BAND = 4e-6f;

// FP32 pair law; returns the force scale s (F = r * s), 0 beyond the cut-off.
// isig2 = 1/sigma_ij^2; e12 = 12*eps_ij (LJ kinds) or eps_ij (repulsion).
template <int KIND>
__device__ __forceinline__ float scale32(float d2, float e12, float sig, float isig2, float third,
                                         bool& near_cut) {
    near_cut = false;
    if constexpr (KIND == KIND_LJCUT || KIND == KIND_LJREPULSE || KIND == KIND_LJATTRACT) {
        const float rsq = d2 * isig2;
        const float cut2 = cut_kind<KIND>() ? third * third : 1.0f;
        if constexpr (cut_kind<KIND>()) near_cut = fabsf(rsq - cut2) <= CUT_BAND * cut2;
        const float ir = __fdividef(1.0f, rsq);
        const float ir3 = ir * ir * ir;   // 1 / rsix
        const float sc = e12 * ir3 * (ir3 - 1.0f) * ir * isig2;   // fmagTimesR / dsq
        // LJAttractCut: no force inside sigma (the force is continuous there)
        if constexpr (KIND == KIND_LJATTRACT)
            if (rsq < 1.0f) return 0.0f;
        return rsq > cut2 ? 0.0f : sc;
    } else {
        if (d2 > sig * sig) return 0.0f;
        const float R = sqrtf(d2);
        const float isig = __fdividef(1.0f, sig);
        // R <= sigma here, but the approximate reciprocal can leave 1 - R/sigma
        // a rounding below zero, where b^1.5 or pow would be NaN
        const float b = fmaxf(1.0f - R * isig, 0.0f);
        float pw;
        if (third == 2.0f) pw = b;
        else if (third == 2.5f) pw = b * sqrtf(b);
        else pw = powf(b, third - 1.0f);
        return e12 * pw * isig * __fdividef(1.0f, R);
    }
}

template <int KIND>
__device__ __forceinline__ float energy32(float d2, float eps, float sig, float third, float m6) {
    if constexpr (KIND == KIND_LJATTRACT) {
        float rsq = d2 / (sig * sig);
        if (eps == 0.0f || rsq > third * third) return 0.0f;
        float e = -eps;
        if (rsq >= 1.0f) {
            float ir3 = 1.0f / (rsq * rsq * rsq);
            float mid = 1.0f - ir3;
            e = eps * (mid * mid - 1.0f);
        }
        return e - m6 * eps;
    } else if constexpr (KIND == KIND_LJCUT || KIND == KIND_LJREPULSE) {
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
        float b = fmaxf(1.0f - R / sig, 0.0f);
        float pw = (third == 2.0f) ? b * b : powf(b, third);
        return eps * pw / third;
    }
}

}  // namespace parm
