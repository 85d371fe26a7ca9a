// bsg_crmath.h -- float exp and log that round correctly to nearest, except
// when the exact result lies within ~2^-44 (relative) of a rounding midpoint.
//
// The reference prices with glibc's expf/logf (blackscholes.c:155, 228, 250
// call exp/log on floats in a C++ translation unit), which are within about
// half an ulp of the exact result: correctly rounded on all but ~0.1 % of
// arguments.  CUDA's accurate expf/logf are within 1-2 ulp, so the
// reference-order pricing mode uses these instead and matches the
// reference's rounding wherever glibc's does.
//
// Both are float-float (pairs of floats) evaluations of published
// table-driven methods (P. T. P. Tang, "Table-driven implementation of the
// exponential function in IEEE floating-point arithmetic", ACM TOMS 15(2),
// 1989, and its logarithm counterpart, ACM TOMS 16(4), 1990), written here
// from the mathematics: Taylor polynomials, error-free transformations
// (Knuth's two-sum, the fma two-product), and tables of 2^(j/32) and
// ln(256/k) computed exactly by gen_crmath_tables.py.
//
// Compiles as CUDA device code and as host C++ (compile the host side with
// -ffp-contract=off: every rounding here is explicit), so that the CPU test
// checks the very code the GPU runs.  No product is rounded and then added
// by a separate operation (each such step is one fma): the packed f32x2
// version of this code (bsg_math.cuh) then rounds exactly as this one, which
// it would not otherwise -- the toolchain fuses an f32x2 multiply into the
// f32x2 add that is its only use.
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "bsg_crmath_tables.h"

#if defined(__CUDACC__)
#define BSG_CR_FN __host__ __device__ __forceinline__
#else
#define BSG_CR_FN inline
#endif

namespace bsg_cr {

struct F2 { float hi, lo; };
struct LogEntry { float c, hi, lo, pad; };  // c = k/256, ln(256/k) = hi + lo

#if defined(__CUDA_ARCH__)
BSG_CR_FN float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
BSG_CR_FN float mul(float a, float b) { return __fmul_rn(a, b); }
BSG_CR_FN float add(float a, float b) { return __fadd_rn(a, b); }
BSG_CR_FN float sub(float a, float b) { return __fsub_rn(a, b); }
BSG_CR_FN float bits_to_float(uint32_t u) { return __uint_as_float(u); }
BSG_CR_FN uint32_t float_to_bits(float f) { return __float_as_uint(f); }
BSG_CR_FN float fallback_exp(float x) { return expf(x); }
BSG_CR_FN float fallback_log(float x) { return logf(x); }
#else
inline float fma_(float a, float b, float c) { return fmaf(a, b, c); }
inline float mul(float a, float b) { return a * b; }
inline float add(float a, float b) { return a + b; }
inline float sub(float a, float b) { return a - b; }
inline float bits_to_float(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
inline uint32_t float_to_bits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
inline float fallback_exp(float x) { return expf(x); }
inline float fallback_log(float x) { return logf(x); }
#endif

// a + b = s + e exactly (Knuth), any magnitudes
BSG_CR_FN F2 two_sum(float a, float b) {
    const float s = add(a, b);
    const float bb = sub(s, a);
    const float e = add(sub(a, sub(s, bb)), sub(b, bb));
    return {s, e};
}
// a + b = s + e exactly when |a| >= |b| (Dekker)
BSG_CR_FN F2 fast_two_sum(float a, float b) {
    const float s = add(a, b);
    return {s, sub(b, sub(s, a))};
}
// a * b = p + e exactly
BSG_CR_FN F2 two_prod(float a, float b) {
    const float p = mul(a, b);
    return {p, fma_(a, b, -p)};
}

// The tables: a device copy (declared in both of nvcc's passes, which both
// must see device variables) and a host copy.
#if defined(__CUDACC__)
static __device__ const F2 kExpTab[32] = {BSG_CR_EXP_TABLE};
static __device__ const LogEntry kLogTab[256] = {BSG_CR_LOG_TABLE};
#endif
static const F2 kExpTabHost[32] = {BSG_CR_EXP_TABLE};
static const LogEntry kLogTabHost[256] = {BSG_CR_LOG_TABLE};
BSG_CR_FN F2 exp_tab(int j) {
#if defined(__CUDA_ARCH__)
    return kExpTab[j];
#else
    return kExpTabHost[j];
#endif
}
BSG_CR_FN LogEntry log_tab(int i) {
#if defined(__CUDA_ARCH__)
    return kLogTab[i];
#else
    return kLogTabHost[i];
#endif
}

// Round-to-nearest-even of |a| < 2^22 and its integer value, by adding and
// subtracting 1.5 * 2^23 (the sum's low mantissa bits are the integer).
constexpr float kShifter = 12582912.0f;
constexpr uint32_t kShifterBits = 0x4B400000u;

// e^x.  Arguments outside [-87, 88.5] (subnormal or overflowing results,
// NaN) go to the platform's expf.
//   x = (32 m + j) ln2/32 + r, |r| <~ ln2/64; e^x = 2^m 2^(j/32) e^r.
//   r = x - n L1 - n L2 - n L3 as a float pair: x - n L1 is exact (L1 has
//   12 bits, |n| < 2^12, the difference has at most 24 bits), n L2 is an
//   exact two-product.  e^r - 1 = r + r^2/2 + r^3 (1/6 + r/24 + r^2/120)
//   (truncation below 2^-48 for |r| <= 0.011), with r^2/2 exact.
BSG_CR_FN float exp(float x) {
    if (!(x >= -87.0f && x <= 88.5f)) return fallback_exp(x);
    const float sh = fma_(x, BSG_CR_INV_L, kShifter);
    const float nf = sub(sh, kShifter);
    const int n = (int)(float_to_bits(sh) - kShifterBits);
    const float r1 = fma_(-nf, BSG_CR_L1, x);
    const F2 p = two_prod(nf, BSG_CR_L2);
    const F2 rs = two_sum(r1, -p.hi);
    const float rh = rs.hi;
    const float rl = fma_(-nf, BSG_CR_L3, sub(rs.lo, p.lo));
    const F2 s2 = two_prod(rh, rh);
    float c = fma_(rh, 1.0f / 120.0f, 1.0f / 24.0f);
    c = fma_(rh, c, 1.0f / 6.0f);
    c = mul(rh, c);
    const F2 q = fast_two_sum(rh, mul(s2.hi, 0.5f));
    const float ql = add(q.lo, add(rl, fma_(s2.lo, 0.5f, fma_(rh, rl, mul(s2.hi, c)))));
    const F2 t = exp_tab(n & 31);
    const F2 tq = two_prod(t.hi, q.hi);
    const F2 s = fast_two_sum(t.hi, tq.hi);
    const float lo = add(s.lo, add(tq.lo, add(t.lo, fma_(t.hi, ql, mul(t.lo, q.hi)))));
    const float y = add(s.hi, lo);
    const int m = n >> 5;  // floor(n / 32): m in [-126, 127] on this domain
    return mul(y, bits_to_float((uint32_t)(m + 127) << 23));
}

// ln x.  Arguments that are not positive normal finite floats (zero,
// subnormal, negative, infinite, NaN) go to the platform's logf.
//   x = 2^e m, m in [1, 2), halved (e + 1) when m >= 1.5; the top 8
//   fraction bits of m pick c = k/256 near 1/m, so that r = m c - 1 is
//   exact (|r| <= 2.5 * 2^-9, the product has <= 24 bits);
//   ln x = e ln2 + ln(256/k) + ln(1 + r),
//   ln(1 + r) = r - r^2/2 + r^3 (1/3 - r/4 + r^2/5) (truncation below 2^-48),
//   summed as float pairs.  For x near 1: e = 0, k = 256, ln(256/k) = 0.
BSG_CR_FN float log(float x) {
    if (!(x >= 1.17549435e-38f && x <= 3.40282347e38f)) return fallback_log(x);
    const uint32_t u = float_to_bits(x);
    const uint32_t i = (u >> 15) & 0xFFu;
    const int e = (int)(u >> 23) - 127 + (int)(i >> 7);
    const float m = bits_to_float((u & 0x7FFFFFu) | (i >= 128 ? 0x3F000000u : 0x3F800000u));
    const LogEntry tab = log_tab((int)i);
    const float r = fma_(m, tab.c, -1.0f);
    const F2 s2 = two_prod(r, r);
    float c = fma_(r, 0.2f, -0.25f);
    c = fma_(r, c, 1.0f / 3.0f);
    c = mul(mul(s2.hi, r), c);
    const F2 a = fast_two_sum(r, mul(s2.hi, -0.5f));
    const float alo = add(a.lo, fma_(s2.lo, -0.5f, c));
    const float ef = sub(bits_to_float(kShifterBits + (uint32_t)e), kShifter);  // (float)e
    const F2 em = two_prod(ef, BSG_CR_LN2M);
    const F2 s1 = two_sum(mul(ef, BSG_CR_LN2H), tab.hi);
    const F2 s2s = two_sum(s1.hi, a.hi);
    const F2 s3 = two_sum(s2s.hi, em.hi);
    const float lo = add(add(add(s1.lo, s2s.lo), s3.lo),
                         add(add(tab.lo, alo), fma_(ef, BSG_CR_LN2L, em.lo)));
    return add(s3.hi, lo);
}

}  // namespace bsg_cr
