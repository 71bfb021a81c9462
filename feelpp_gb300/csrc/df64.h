// Double-float ("df64") arithmetic: a value is the unevaluated sum hi + lo of
// two binary32 numbers (|lo| <= ulp(hi)), about 48 significant bits.
//
// Why: on GB300 the FP64 pipe runs at 1/71 of the FP32 rate (1.0 vs 71.9
// TFLOP/s measured) and f64<->f32 conversions occupy that same pipe. The
// FP64-accurate assembly therefore computes with error-free transformations
// on the FP32 pipes (Dekker / Knuth TwoSum and an FMA-based TwoProduct), and
// converts between double and df64 with integer bit manipulation.
//
// All operations use explicitly rounded intrinsics on the device (never
// contracted or re-associated by the compiler); on the host the same code runs
// with plain float operations and must be compiled with -ffp-contract=off.
//
// Accuracy (unit roundoff u = 2^-24; bounds checked against exact rationals by
// tests/test_df64.py, which also covers the conversions below):
//   two_sum, two_prod     exact
//   df_add (sloppy)       |err| <= 2u^2 (|x| + |y|)
//   df_mul                |err| <= 4u^2 |x y|
//   df_recip              |err| <= 2^-46 |1/x|  (one Newton step from the rounded binary32 reciprocal)
//   d2df                  |err| <= 2^-48 |x|   for 2^-100 <= |x| <= 2^127 (both halves normal)
//   df2d                  |err| <= 2^-53 |hi + lo|
#pragma once
#include <cstdint>
#include <cstring>
#include <cmath>

#if defined(__CUDACC__)
#define FGPU_HD __host__ __device__ __forceinline__
#else
#define FGPU_HD inline
#endif

namespace fgpu {

struct df {
    float hi, lo;
};

FGPU_HD float f_add(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
FGPU_HD float f_sub(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
FGPU_HD float f_mul(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
FGPU_HD float f_fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}
FGPU_HD uint32_t f_bits(float x) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(x);
#else
    uint32_t u;
    std::memcpy(&u, &x, 4);
    return u;
#endif
}
FGPU_HD float f_from_bits(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float x;
    std::memcpy(&x, &u, 4);
    return x;
#endif
}
FGPU_HD uint64_t d_bits(double x) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    std::memcpy(&u, &x, 8);
    return u;
#endif
}
FGPU_HD double d_from_bits(uint64_t u) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double x;
    std::memcpy(&x, &u, 8);
    return x;
#endif
}
FGPU_HD int clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return __clzll((long long)x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

// Knuth TwoSum: s + e == a + b exactly.
FGPU_HD df two_sum(float a, float b) {
    float s = f_add(a, b);
    float bb = f_sub(s, a);
    float e = f_add(f_sub(a, f_sub(s, bb)), f_sub(b, bb));
    return {s, e};
}
// Dekker FastTwoSum, requires |a| >= |b| (or a == 0).
FGPU_HD df quick_two_sum(float a, float b) {
    float s = f_add(a, b);
    float e = f_sub(b, f_sub(s, a));
    return {s, e};
}
FGPU_HD df df_add(df x, df y) {
    df s = two_sum(x.hi, y.hi);
    float e = f_add(s.lo, f_add(x.lo, y.lo));
    return quick_two_sum(s.hi, e);
}
FGPU_HD df df_neg(df x) { return {-x.hi, -x.lo}; }
FGPU_HD df df_sub(df x, df y) { return df_add(x, df_neg(y)); }
FGPU_HD df df_mul(df x, df y) {
    float p = f_mul(x.hi, y.hi);
    float e = f_fma(x.hi, y.hi, -p);
    e = f_fma(x.hi, y.lo, e);
    e = f_fma(x.lo, y.hi, e);
    return quick_two_sum(p, e);
}
// x * 2^k for a small exact power of two given as a float
FGPU_HD df df_scale(df x, float pow2) { return {f_mul(x.hi, pow2), f_mul(x.lo, pow2)}; }
// 1 / x: Newton step in df64 from the correctly rounded binary32 reciprocal.
FGPU_HD df df_recip(df x) {
#if defined(__CUDA_ARCH__)
    float r = __frcp_rn(x.hi);
#else
    float r = 1.0f / x.hi;
#endif
    df xr = df_mul(x, df{r, 0.0f});
    df e = df_sub(df{1.0f, 0.0f}, xr);
    df t = df_mul(df{r, 0.0f}, e);
    return df_add(df{r, 0.0f}, t);
}

// double -> df64 with integer operations only. Zero, subnormal doubles and
// magnitudes below 2^-126 map to 0; magnitudes above the binary32 range map to inf.
FGPU_HD df d2df(double x) {
    uint64_t b = d_bits(x);
    uint32_t sign = (uint32_t)(b >> 63);
    int e = (int)((b >> 52) & 0x7FF);
    uint64_t m = b & 0xFFFFFFFFFFFFFull;
    int fe = e - 1023 + 127;
    if (e == 0 || fe <= 0) return {sign ? -0.0f : 0.0f, 0.0f};
    if (fe >= 255) return {f_from_bits((sign << 31) | 0x7F800000u), 0.0f};
    float hi = f_from_bits((sign << 31) | ((uint32_t)fe << 23) | (uint32_t)(m >> 29));
    uint32_t rest = (uint32_t)(m & ((1ull << 29) - 1));      // value rest * 2^(e - 1075)
    float lo = 0.0f;
    if (rest) {
        int pe = e - 1075 + 127;                               // biased exponent of 2^(e - 1075)
        float r = (float)rest;                                 // rounds 29 -> 24 bits
        if (pe >= 1) {
            lo = f_mul(r, f_from_bits((uint32_t)pe << 23));
        } else {
            lo = std::ldexp(r, e - 1075);
        }
        if (sign) lo = -lo;
    }
    return quick_two_sum(hi, lo);
}

// df64 -> double with integer operations only (hi normal or zero; lo below 2^-126 ignored).
FGPU_HD double df2d(df x) {
    uint32_t hb = f_bits(x.hi);
    int he = (int)((hb >> 23) & 0xFF);
    if (he == 0) return (hb >> 31) ? -0.0 : 0.0;
    if (he == 255) return (hb >> 31) ? -INFINITY : INFINITY;
    int64_t mh = (int64_t)((hb & 0x7FFFFFu) | 0x800000u);     // value mh * 2^(he - 150)
    if (hb >> 31) mh = -mh;
    uint32_t lb = f_bits(x.lo);
    int le = (int)((lb >> 23) & 0xFF);
    int64_t M = mh * ((int64_t)1 << 29);                      // value M * 2^(he - 179)
    if (le != 0 && le != 255) {
        int64_t ml = (int64_t)((lb & 0x7FFFFFu) | 0x800000u);
        if (lb >> 31) ml = -ml;
        int d = he - le;
        if (d <= 29) M += ml * ((int64_t)1 << (29 - d));
        else if (d - 29 < 63) M += ml >> (d - 29);
    }
    uint64_t sign = 0;
    if (M < 0) { sign = 1; M = -M; }
    if (M == 0) return 0.0;
    uint64_t U = (uint64_t)M;
    int top = 63 - clz64(U);                                  // highest set bit
    int shift = top - 52;
    if (shift > 0) {
        uint64_t half = (uint64_t)1 << (shift - 1);
        U = (U + half) >> shift;
        if (U >> 53) { U >>= 1; ++shift; }
    } else if (shift < 0) {
        U <<= -shift;
    }
    int64_t de = (int64_t)he - 179 + shift + 52 + 1023;
    return d_from_bits((sign << 63) | ((uint64_t)de << 52) | (U & 0xFFFFFFFFFFFFFull));
}

}  // namespace fgpu
