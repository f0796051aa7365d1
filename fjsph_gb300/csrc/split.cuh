/*
 * split.cuh -- FP64 -> FP32 rounding in integer arithmetic.
 *
 * On this GPU the FP64 pipe issues a warp instruction every 16 cycles per SM, and conversions
 * between FP64 and FP32 run there too; the per-particle kernels that write the split-precision
 * inputs (hi = fl32(x), lo = fl32(x - hi) for every coordinate and velocity component) spent
 * most of their time on those conversions.  These helpers compute the same IEEE round-to-
 * nearest-even results from the bit pattern with 32/64-bit integer operations and one
 * int32 -> FP32 conversion.  Outside the exponent range they cover (zero, subnormals, very small
 * or very large magnitudes, NaN / infinity) they fall back to the conversions.
 *
 * Plain C++ with CUDA decorations: the host compiles the same code for its exhaustive check
 * against the compiler's conversions.
 */
#pragma once

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define FJSPH_HD __host__ __device__ __forceinline__
#else
#define FJSPH_HD inline
#endif

namespace fjsph {

FJSPH_HD uint64_t f64_bits(double x) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    memcpy(&u, &x, sizeof u);
    return u;
#endif
}

FJSPH_HD float f32_from_bits(uint32_t b) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(b);
#else
    float f;
    memcpy(&f, &b, sizeof f);
    return f;
#endif
}

FJSPH_HD uint32_t f32_bits(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t b;
    memcpy(&b, &f, sizeof b);
    return b;
#endif
}

FJSPH_HD double f64_from_bits(uint64_t u) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    double x;
    memcpy(&x, &u, sizeof x);
    return x;
#endif
}

/* (double)f, exact: zeros and normal numbers by moving the fields, the rest by the conversion */
FJSPH_HD double to_f64(float f) {
    const uint32_t b = f32_bits(f);
    const uint32_t e = (b >> 23) & 0xFFu;
    const uint64_t sign = (uint64_t)(b & 0x80000000u) << 32;
    if ((b & 0x7FFFFFFFu) == 0u) return f64_from_bits(sign);
    if (e == 0u || e == 0xFFu) return (double)f;
    return f64_from_bits(sign | ((uint64_t)(e + 896u) << 52) | ((uint64_t)(b & 0x7FFFFFu) << 29));
}

/* Biased FP64 exponents handled by the integer path: |x| in [2^-63, 2^127).  Below, the low
 * part's scale 2^(e - 1075) would leave the FP32 normal range; above, the rounding may overflow
 * to infinity (left to the conversions). */
constexpr int kSplitEMin = 960, kSplitEMax = 1149;

/* The 24-bit significand of x rounded to nearest even (r may reach 2^24), the 29 dropped bits
 * and whether it rounded up.  Requires a normal x. */
struct Rounded24 {
    uint32_t r, rem, up;
};
FJSPH_HD Rounded24 round24(uint64_t u) {
    const uint64_t M = (u & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    Rounded24 q;
    q.r = (uint32_t)(M >> 29);
    q.rem = (uint32_t)(M & 0x1FFFFFFFu);
    q.up = (q.rem > 0x10000000u || (q.rem == 0x10000000u && (q.r & 1u))) ? 1u : 0u;
    q.r += q.up;
    return q;
}

/* FP32 bits of sign * r * 2^(e - 1046), r in [2^23, 2^24]: r = 2^24 carries into the exponent. */
FJSPH_HD uint32_t f32_bits_of(uint32_t sign, int e, uint32_t r) {
    const int eh = e - 896;
    return r == (1u << 24) ? (sign | ((uint32_t)(eh + 1) << 23)) : (sign | ((uint32_t)eh << 23) | (r & 0x7FFFFFu));
}

/* fl32(x), round to nearest even */
FJSPH_HD float to_f32(double x) {
    const uint64_t u = f64_bits(x);
    const int e = (int)((u >> 52) & 0x7FF);
    if (e < kSplitEMin || e > kSplitEMax) return (float)x;
    const Rounded24 q = round24(u);
    return f32_from_bits(f32_bits_of((uint32_t)(u >> 32) & 0x80000000u, e, q.r));
}

/* hi = fl32(x), lo = fl32(x - hi) (x - hi is exact in FP64) */
FJSPH_HD void split_f32(double x, float &hi, float &lo) {
    const uint64_t u = f64_bits(x);
    const int e = (int)((u >> 52) & 0x7FF);
    if (e < kSplitEMin || e > kSplitEMax) {
        hi = (float)x;
        lo = (float)(x - (double)hi);
        return;
    }
    const uint32_t sign = (uint32_t)(u >> 32) & 0x80000000u;
    const Rounded24 q = round24(u);
    hi = f32_from_bits(f32_bits_of(sign, e, q.r));
    /* x - hi = +-(rem - up 2^29) 2^(e - 1075): an integer of at most 29 bits, rounded once by the
     * int32 -> FP32 conversion, then scaled exactly by a power of two */
    const int32_t d = (int32_t)q.rem - (int32_t)(q.up << 29);
    lo = (float)(sign ? -d : d) * f32_from_bits((uint32_t)(e - 1075 + 127) << 23); /* x - hi = 0 is +0 */
}

} // namespace fjsph
