// Conversions between FP32 and FP64 on the bit patterns, with integer
// instructions.  GB300 runs FP64 arithmetic, and the conversion instructions
// that take or give an FP64 value, at a small fraction of its FP32 rate; the
// per-atom update of the mixed-precision step converts nine values per atom
// and is bound by that pipe.  Both functions return exactly what the
// conversion instruction returns (IEEE 754: float to double is exact, double
// to float rounds to nearest, ties to even); values outside the common case
// (zero, subnormal results or inputs, overflow, inf, NaN) take the
// instruction itself.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define PARM_FPB_HD __host__ __device__ __forceinline__
#else
#define PARM_FPB_HD inline
#endif

namespace parm {

PARM_FPB_HD uint32_t fpb_f2u(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
#endif
}

PARM_FPB_HD float fpb_u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    std::memcpy(&f, &u, 4);
    return f;
#endif
}

PARM_FPB_HD double fpb_hilo2d(uint32_t hi, uint32_t lo) {
#if defined(__CUDA_ARCH__)
    return __hiloint2double((int)hi, (int)lo);
#else
    const uint64_t b = ((uint64_t)hi << 32) | lo;
    double d;
    std::memcpy(&d, &b, 8);
    return d;
#endif
}

PARM_FPB_HD void fpb_d2hilo(double d, uint32_t& hi, uint32_t& lo) {
#if defined(__CUDA_ARCH__)
    hi = (uint32_t)__double2hiint(d);
    lo = (uint32_t)__double2loint(d);
#else
    uint64_t b;
    std::memcpy(&b, &d, 8);
    hi = (uint32_t)(b >> 32);
    lo = (uint32_t)b;
#endif
}

// (double)f: a normal float moves its exponent from bias 127 to bias 1023
// and its 23 fraction bits to the top of the 52
PARM_FPB_HD double f2d_bits(float f) {
    const uint32_t b = fpb_f2u(f);
    const uint32_t e = (b >> 23) & 0xFFu;
    if (e - 1u < 254u) {
        const uint32_t hi = (b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7FFFFFu) >> 3);
        return fpb_hilo2d(hi, b << 29);
    }
    return (double)f;
}

// (float)d: a double whose float result is normal keeps its top 23 fraction
// bits, rounded to nearest (ties to even) on the 29 dropped ones; a carry out
// of the fraction moves into the exponent, as the rounding requires
PARM_FPB_HD float d2f_bits(double d) {
    uint32_t hi, lo;
    fpb_d2hilo(d, hi, lo);
    const uint32_t e = (hi >> 20) & 0x7FFu;
    if (e - 897u < 254u) {
        uint32_t f = (hi & 0x80000000u) | ((e - 896u) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29);
        const uint32_t rem = lo & 0x1FFFFFFFu;
        f += (rem > 0x10000000u || (rem == 0x10000000u && (f & 1u))) ? 1u : 0u;
        return fpb_u2f(f);
    }
    return (float)d;
}

PARM_FPB_HD float fpb_i2f(int32_t i) {
#if defined(__CUDA_ARCH__)
    return __int2float_rn(i);
#else
    return (float)i;
#endif
}

PARM_FPB_HD float fpb_fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}

PARM_FPB_HD float fpb_sub(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}

// The fine part x - X of a position against its coarse point X (a float,
// a multiple of 1/8 within about 1/4 of x), in FP32 without FP64 arithmetic:
// x = xh + r with xh = (float)x (the rounding above) and r the 29 dropped
// fraction bits (signed by the rounding direction: |r| <= ulp(xh) / 2, an
// integer count of x's ulps, scaled by a power of two), then
// (xh - X) + r with one rounding (a fused multiply-add).  xh - X is exact
// when X and xh are within a factor of two (the rule of Sterbenz), so the
// result is (float)(x - X) but for a rare double rounding near a tie (r is
// itself rounded to 24 bits); near the origin, where X may lie in another
// binade, xh - X can round too.  Either way the result is within one ulp of
// (float)(x - X).  Outside 2^-74 <= |x| < 2^127 the FP64 subtraction is
// taken.
PARM_FPB_HD float fine_bits(double x, float X) {
    uint32_t hi, lo;
    fpb_d2hilo(x, hi, lo);
    const uint32_t e = (hi >> 20) & 0x7FFu;
    if (e - 949u < 200u) {
        uint32_t f = (hi & 0x80000000u) | ((e - 896u) << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29);
        const uint32_t rem = lo & 0x1FFFFFFFu;
        const bool up = rem > 0x10000000u || (rem == 0x10000000u && (f & 1u));
        f += up ? 1u : 0u;
        // |x| - |xh| in units of 2^(e - 1075), then the sign of x
        int32_t r = up ? (int32_t)rem - 0x20000000 : (int32_t)rem;
        if (hi & 0x80000000u) r = -r;
        return fpb_fma(fpb_i2f(r), fpb_u2f((e - 948u) << 23), fpb_sub(fpb_u2f(f), X));
    }
    return d2f_bits(x - f2d_bits(X));
}

}  // namespace parm
