// bsg_swmath.h -- double-precision elementary functions of the swaption
// Monte Carlo: the normal variates (Box-Muller evaluated from the bits of
// the uniforms with table-driven -2 ln u and sin/cos(2 pi u)) and the
// exponential of the discount factors.
//
// The uniforms are u = (2k + 1) 2^-53 for a 52-bit integer k (the grid of
// midpoints in (0, 1)); a pair (u1, u2) gives z0 = sqrt(-2 ln u1) cos(2 pi u2)
// and z1 = sqrt(-2 ln u1) sin(2 pi u2).  Both functions start from k itself,
// so neither the uniform nor the angle is ever rounded:
//
//  -2 ln u: u = 2^e m with m in [1, 2) read off k's bits; m = F (1 + r) with
//    F = 1 + j/128 the nearest 1/128 step (|r| <= 2^-8); -2 ln u =
//    -2 (e ln 2 + ln F) + W(r'), r' = -2 r = (m - F)(-2/F), W(r') =
//    -2 ln(1 - r'/2) = sum_k 2^(1-k) r'^k / k to k = 7.  For F >= 1.5 the
//    table holds ln(F/2) and e is one larger, so that u near 1 (e = -1, F =
//    2) gives -2 ln u = W(r') exactly as small as it is (no cancellation).
//    This is the table-driven logarithm of P. T. P. Tang, ACM TOMS 16(4),
//    1990, written here from the mathematics (Taylor series of ln(1 + r)).
//  sin/cos(2 pi u): j = the nearest multiple of 1/256 to u, u = j/256 +
//    x 2^-53 with the integer x = 2k + 1 - j 2^45 (|x| <= 2^44 + 1), phi =
//    x (2 pi 2^-53) (|phi| <= pi/256); the angle-addition formulas combine
//    the table's sin/cos(2 pi j/256) with Taylor polynomials of sin phi (to
//    phi^7) and cos phi - 1 (to phi^6).
//  e^x: x = (64 m + j) ln2/64 + r with k = 64 m + j the integer nearest
//    64 x / ln 2 (|r| <= ln2/128), e^x = 2^m 2^(j/64) (1 + p(r)), p the
//    Taylor polynomial of e^r - 1 to r^6; ln2/64 in two parts so that r is
//    exact to far below its ulp (P. T. P. Tang, ACM TOMS 15(2), 1989).
//    Arguments of magnitude 700 or more (and NaN) go to the platform's exp.
//
// Every operation is an explicitly rounded IEEE double operation (add, mul,
// fma, sqrt) or integer work, so the host build of this header (compile it
// with -ffp-contract=off) gives the same bits as the GPU; the CPU test
// checks the very code the GPU runs.  Errors: within a few ulp of the exact
// values (the test states the bounds), at about half the double-precision
// work of calling log, sqrt, sincospi and exp.
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "bsg_swmath_tables.h"

#if defined(__CUDACC__)
#define BSG_SW_FN __host__ __device__ __forceinline__
#else
#define BSG_SW_FN inline
#endif

namespace bsg_sw {

struct alignas(16) LogEntry { double neg2_inv_f, neg2_ln_f; };
struct alignas(16) Angle { double s, c; };

// 7,184 bytes: the kernels copy it into shared memory once per block.
struct Tables {
    LogEntry lg[129];
    double e2[64];   // 2 i ln 2
    Angle ang[256];
    double e64[64];  // 2^(j/64)
};

#if defined(__CUDA_ARCH__)
BSG_SW_FN double fma_(double a, double b, double c) { return __fma_rn(a, b, c); }
BSG_SW_FN double mul(double a, double b) { return __dmul_rn(a, b); }
BSG_SW_FN double add(double a, double b) { return __dadd_rn(a, b); }
BSG_SW_FN double sqrt_(double a) { return __dsqrt_rn(a); }
BSG_SW_FN double from_bits(uint64_t u) { return __longlong_as_double((long long)u); }
BSG_SW_FN int clz64(uint64_t v) { return __clzll((long long)v); }
BSG_SW_FN uint64_t to_bits(double d) { return (uint64_t)__double_as_longlong(d); }
BSG_SW_FN double exp_fallback(double x) { return exp(x); }
#else
inline double fma_(double a, double b, double c) { return fma(a, b, c); }
inline double mul(double a, double b) { return a * b; }
inline double add(double a, double b) { return a + b; }
inline double sqrt_(double a) { return sqrt(a); }
inline double from_bits(uint64_t u) { double d; memcpy(&d, &u, 8); return d; }
inline int clz64(uint64_t v) { return __builtin_clzll(v); }
inline uint64_t to_bits(double d) { uint64_t u; memcpy(&u, &d, 8); return u; }
inline double exp_fallback(double x) { return exp(x); }
#endif

// The 52-bit integer k of a uniform from two 32-bit random words (the top
// 20 bits of a, all of b).
BSG_SW_FN uint64_t unit_bits(uint32_t a, uint32_t b) { return ((uint64_t)(a >> 12) << 32) | b; }

// -2 ln u for u = (2k + 1) 2^-53, k < 2^52: a value in (0, 73.5].
BSG_SW_FN double neg2_ln_unit(const Tables& t, uint64_t k) {
    const uint64_t v = 2 * k + 1;                        // u = v 2^-53, v odd
    const int lz = clz64(v);                             // 11..63
    const uint64_t frac = (v << (lz - 11)) & ((1ull << 52) - 1);
    const int j = (int)((frac + (1ull << 44)) >> 45);    // nearest 1/128: 0..128
    const double m = from_bits(0x3FF0000000000000ull | frac);              // [1, 2)
    const double f = from_bits(0x3FF0000000000000ull + ((uint64_t)j << 45));  // 1 + j/128
    // u = 2^e m with e = 10 - lz; the table's entry for j >= 64 is ln(F/2),
    // so the power of two taken out is e + 1 there: -(e + [j >= 64]) >= 0
    const int ne = lz - 10 - (j >= 64 ? 1 : 0);          // 0..53
    const LogEntry le = t.lg[j];
    const double rp = mul(add(m, -f), le.neg2_inv_f);    // r' = -2 (m - F)/F, m - F exact
    double q = 1.0 / 448;                                // W(r') = r' + r'^2 (1/4 + r'/12 + ...)
    q = fma_(q, rp, 1.0 / 192);
    q = fma_(q, rp, 1.0 / 80);
    q = fma_(q, rp, 1.0 / 32);
    q = fma_(q, rp, 1.0 / 12);
    q = fma_(q, rp, 0.25);
    const double wr = fma_(mul(rp, rp), q, rp);
    return add(add(t.e2[ne], le.neg2_ln_f), wr);
}

// sin(2 pi u) and cos(2 pi u) for u = (2k + 1) 2^-53, k < 2^52.
BSG_SW_FN void sincos_2pi_unit(const Tables& t, uint64_t k, double* s, double* c) {
    const int j = (int)((k + (1ull << 43)) >> 44);       // nearest 1/256: 0..256
    const int64_t x = (int64_t)(2 * k + 1) - ((int64_t)j << 45);  // |x| <= 2^44 + 1
    // x as a double: 1.5 2^52 + x has x in its low bits (|x| < 2^51)
    const double xd = add(from_bits(0x4338000000000000ull + (uint64_t)x), -6755399441055744.0);
    const double ph = mul(xd, BSG_SW_TWO_PI_ULP);        // |phi| <= pi/256
    const double p2 = mul(ph, ph);
    double ps = fma_(-1.0 / 5040, p2, 1.0 / 120);
    ps = fma_(ps, p2, -1.0 / 6);
    const double sp = fma_(mul(p2, ph), ps, ph);         // sin phi
    double pc = fma_(-1.0 / 720, p2, 1.0 / 24);
    pc = fma_(pc, p2, -0.5);
    const double cm = mul(p2, pc);                       // cos phi - 1
    const Angle a = t.ang[j & 255];
    *s = add(a.s, fma_(a.c, sp, mul(a.s, cm)));
    *c = add(a.c, fma_(-a.s, sp, mul(a.c, cm)));
}

// Normal variates z0, z1 from four random words: u1 from (w0, w1), u2 from (w2, w3).
BSG_SW_FN void normal_pair(const Tables& t, uint32_t w0, uint32_t w1, uint32_t w2, uint32_t w3,
                           double* z0, double* z1) {
    const double r = sqrt_(neg2_ln_unit(t, unit_bits(w0, w1)));
    double s, c;
    sincos_2pi_unit(t, unit_bits(w2, w3), &s, &c);
    *z0 = mul(r, c);
    *z1 = mul(r, s);
}

// e^x; for |x| >= 700 or NaN, the platform's exp.
BSG_SW_FN double exp_(const Tables& t, double x) {
    if ((to_bits(x) & 0x7FFFFFFFFFFFFFFFull) >= 0x4085E00000000000ull) return exp_fallback(x);  // 700
    const double tm = fma_(x, BSG_SW_INV_L, 6755399441055744.0);  // 1.5 2^52 + k
    const double kd = add(tm, -6755399441055744.0);
    const int k = (int)(uint32_t)to_bits(tm);                      // |k| < 2^16
    double r = fma_(-kd, BSG_SW_L1, x);
    r = fma_(-kd, BSG_SW_L2, r);
    double q = 1.0 / 720;
    q = fma_(q, r, 1.0 / 120);
    q = fma_(q, r, 1.0 / 24);
    q = fma_(q, r, 1.0 / 6);
    q = fma_(q, r, 0.5);
    const double p = fma_(mul(r, r), q, r);                        // e^r - 1
    const double tj = t.e64[k & 63];
    const double y = fma_(tj, p, tj);                              // in [0.99, 2.01)
    return from_bits(to_bits(y) + ((uint64_t)(int64_t)(k >> 6) << 52));
}

}  // namespace bsg_sw

// The tables' initializer: `const bsg_sw::Tables t = BSG_SW_TABLES;`
#define BSG_SW_TABLES \
    {{BSG_SW_LOG_TABLE}, {BSG_SW_EXP2_TABLE}, {BSG_SW_ANGLE_TABLE}, {BSG_SW_EXP_TABLE}}
