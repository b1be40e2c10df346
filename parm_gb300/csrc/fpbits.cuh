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

}  // namespace parm
