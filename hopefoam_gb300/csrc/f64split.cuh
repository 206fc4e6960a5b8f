// f64split.cuh -- FP64 -> FP32 differences without the FP64 pipe.
//
// GB300 retires two FP64 operations per clock per SM, and a warp instruction
// holds that pipe for its full width.  The split-precision Euler stage needs,
// for every staged value and every neighbour trace value, d = q - b rounded
// to FP32, with q the FP64 state and b an FP32 reference value.  Done as
// (float)(q - (double)b) that is two FP64 operations per value.  Here q is
// taken apart with integer operations instead:
//   q = qh + ql,  qh = q with its significand truncated to 24 bits (an FP32
//                      value, exact),
//                 ql = the 29 dropped significand bits, times 2^(e - 1075),
//                      converted to FP32 (one integer-to-float conversion),
//   d = (qh - b) + ql   in FP32.
// When qh and b are within a factor of two, qh - b is exact (Sterbenz) and d
// is the correctly rounded difference up to the rounding of ql (at most
// 2^-46 |q|); otherwise the two FP32 roundings give at most ~1 ulp of d.
// |q| < 2^-126 (including zero) is taken as 0 (an absolute error below
// 1.2e-38); |q| >= 2^128, infinities and NaN take the FP64 route, so they
// propagate exactly as before.
//
// Compiles for the host too (the bit logic is checked against FP64 there).
#pragma once

#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define F64S_HD __host__ __device__ __forceinline__
#else
#define F64S_HD inline
#endif

namespace f64s {

F64S_HD uint32_t f_bits(float x) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(x);
#else
    uint32_t u;
    memcpy(&u, &x, 4);
    return u;
#endif
}

F64S_HD float bits_f(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float x;
    memcpy(&x, &u, 4);
    return x;
#endif
}

F64S_HD void d_words(double q, uint32_t& hi, uint32_t& lo) {
#ifdef __CUDA_ARCH__
    hi = (uint32_t)__double2hiint(q);
    lo = (uint32_t)__double2loint(q);
#else
    uint64_t u;
    memcpy(&u, &q, 8);
    hi = (uint32_t)(u >> 32);
    lo = (uint32_t)u;
#endif
}

F64S_HD float u32_to_f(uint32_t m) {
#ifdef __CUDA_ARCH__
    return __uint2float_rn(m);
#else
    return (float)m;
#endif
}

// q truncated to FP32 (toward zero); 0 for |q| < 2^-126; the FP64 conversion
// for |q| >= 2^128, infinities and NaN
F64S_HD float trunc_f32(double q) {
    uint32_t H, L;
    d_words(q, H, L);
    const uint32_t e = (H >> 20) & 0x7FFu;
    if (e > 1150u) return (float)q;
    const uint32_t qh = (H & 0x80000000u) | ((e - 896u) << 23) | ((H & 0xFFFFFu) << 3) | (L >> 29);
    return e < 897u ? 0.f : bits_f(qh);
}

// q - b rounded to FP32 (see the header)
F64S_HD float minus_f32(double q, float b) {
    uint32_t H, L;
    d_words(q, H, L);
    const uint32_t e = (H >> 20) & 0x7FFu;
    if (e > 1150u) return (float)(q - (double)b);
    const uint32_t sign = H & 0x80000000u;
    const bool tiny = e < 897u;
    const float qh = tiny ? 0.f : bits_f(sign | ((e - 896u) << 23) | ((H & 0xFFFFFu) << 3) | (L >> 29));
    // weight of the FP64 significand's last bit, 2^(e - 1075), as an FP32 power of two
    const float scale = e >= 949u ? bits_f((e - 948u) << 23) : 0.f;
    const float ql = bits_f(f_bits(u32_to_f(L & 0x1FFFFFFFu) * scale) | sign);
    return (qh - b) + ql;
}

// x widened to FP64 exactly, from its bits (the FP32 -> FP64 conversion
// instruction occupies the FP64 pipe); zero, subnormal, infinite and NaN
// inputs take the conversion instruction
F64S_HD double widen(float x) {
    const uint32_t u = f_bits(x);
    const uint32_t e = (u >> 23) & 0xFFu;
    if (e == 0u || e == 255u) return (double)x;
    const uint32_t hi = (u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7FFFFFu) >> 3);
    const uint32_t lo = u << 29;
#ifdef __CUDA_ARCH__
    return __hiloint2double((int)hi, (int)lo);
#else
    const uint64_t b = ((uint64_t)hi << 32) | lo;
    double d;
    memcpy(&d, &b, 8);
    return d;
#endif
}

}  // namespace f64s
