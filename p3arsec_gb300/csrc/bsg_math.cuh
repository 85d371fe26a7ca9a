// bsg_math.cuh -- per-option Black-Scholes arithmetic for the sm_103a kernels.
//
// One European option, no dividends: BlkSchlsEqEuroNoDiv and its polynomial
// CNDF (parsec-ff/pkgs/apps/blackscholes/src/blackscholes.c:126-258).  Four
// evaluations of the same formula:
//
//   price_fast      compensated FP32 (production): SFU approximations only
//                   where their error cancels, error-free transformations
//                   where it does not (see the notes on each step).
//   price_sfu_ref   the reference's operation order with SFU intrinsics.
//   price_libm_ref  the reference's operation order with correctly rounded
//                   exp/log (float-float, bsg_crmath.h), IEEE division and
//                   square root, and the reference's double-literal
//                   products emulated in FP32: the reference's rounding
//                   wherever glibc's expf/logf round correctly.
//   price_fp64      the same formula in double (validation oracle).
//
// Every function here is branch-free per option apart from selects, and uses
// only explicit intrinsics (__fmaf_rn etc.) in the FP32 paths, so the result
// for an option never depends on where or with what it is priced.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "bsg_crmath.h"
#include "bsg_internal.h"

namespace bsg {

// ---------------------------------------------------------------- constants
// A&S 26.2.17 coefficients as the reference writes them (blackscholes.c:159-173).
#define BSG_C0 0.2316419
#define BSG_C1 0.319381530
#define BSG_C2 (-0.356563782)
#define BSG_C3 1.781477937
#define BSG_C4 (-1.821255978)
#define BSG_C5 1.330274429
#define BSG_INV_SQRT_2PI 0.39894228040143270286
#define BSG_LOG2E 1.4426950408889634074
#define BSG_LN2 0.69314718055994530942

// ------------------------------------------------------ SFU approximations
// PTX approximate instructions (MUFU).  .ftz: denormal inputs and results
// are flushed to zero, which only affects exp(-x^2/2) for |x| > 13, where the
// CNDF tail is below float resolution anyway.
__device__ __forceinline__ float ex2_approx(float a) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
}
__device__ __forceinline__ float lg2_approx(float a) {
    float r;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
}
__device__ __forceinline__ float rcp_approx(float a) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
}
__device__ __forceinline__ float rsqrt_approx(float a) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
}
__device__ __forceinline__ float sqrt_approx(float a) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
    return r;
}

// float-float split of a double constant: hi + lo == c to ~2^-48.
struct FF { float hi, lo; };
__host__ __device__ constexpr FF split(double c) {
    return FF{(float)c, (float)(c - (double)(float)c)};
}

// ---------------------------------------------------------- compensated path
//
// CNDF tail Q(x) = phi(x) * P(k(x)) for x >= 0, where phi(x) = exp(-x^2/2)/
// sqrt(2 pi), k = 1/(1 + c0 x) and P(k) = k (c1 + c2 k + c3 k^2 + c4 k^3 +
// c5 k^4).  N(x) = 1 - Q(x) for x >= 0 and Q(-x) for x < 0.
//
// Error design (max |price error| is S*Q*relerr(Q) where two ~80-sized
// terms partially cancel, so Q needs ~1e-7 relative accuracy):
//  * k is refined by one Newton step and its residual against the exact
//    1 + c0 x (c0 and y carried as float-float) is kept as k_lo.
//  * The inner polynomial is re-expanded around k = 1 in w = 1 - k = c0 x k:
//    inner(1 - w) = b0 + b1 w + ... + b4 w^4 with b_j = (-1)^j sum_i C(i,j)
//    c_{i+1} (exact algebra on the same polynomial).  Where Q is large, w is
//    small and this Horner has almost no cancellation.
//  * exp(-x^2/2) = 2^a with a = -x^2 log2(e)/2 carried as float-float; the
//    SFU evaluates 2^a_hi and the residual multiplies in as (1 + a_lo ln 2).
//  * 1/sqrt(2 pi) is applied as a float-float constant.
__device__ __forceinline__ float tail_q(float x) {
    constexpr FF c0 = split(BSG_C0);
    constexpr FF isp = split(BSG_INV_SQRT_2PI);
    constexpr float b0 = (float)(BSG_C1 + BSG_C2 + BSG_C3 + BSG_C4 + BSG_C5);
    constexpr float b1 = (float)(-(BSG_C2 + 2 * BSG_C3 + 3 * BSG_C4 + 4 * BSG_C5));
    constexpr float b2 = (float)(BSG_C3 + 3 * BSG_C4 + 6 * BSG_C5);
    constexpr float b3 = (float)(-(BSG_C4 + 4 * BSG_C5));
    constexpr float b4 = (float)BSG_C5;
    constexpr float half_log2e = (float)(-0.5 * BSG_LOG2E);
    constexpr float ln2 = (float)BSG_LN2;

    // Beyond x = 40 the tail is 0 in float; clamping keeps inf from turning
    // the error-free transformations into NaN (NaN still propagates).
    x = (x > 40.0f) ? 40.0f : x;

    const float cx = __fmul_rn(c0.hi, x);
    const float y = __fmaf_rn(c0.hi, x, 1.0f);
    const float y_lo = __fmaf_rn(c0.lo, x, __fmaf_rn(c0.hi, x, 1.0f - y));
    const float k0 = rcp_approx(y);
    const float k = __fmaf_rn(k0, __fmaf_rn(-y, k0, 1.0f), k0);
    const float res = __fmaf_rn(-y_lo, k, __fmaf_rn(-y, k, 1.0f));
    const float k_lo = __fmul_rn(k, res);

    const float w = __fmul_rn(cx, k);
    float in = __fmaf_rn(w, b4, b3);
    in = __fmaf_rn(w, in, b2);
    in = __fmaf_rn(w, in, b1);
    in = __fmaf_rn(w, in, b0);
    const float p = __fmaf_rn(in, k_lo, __fmul_rn(in, k));

    const float xx = __fmul_rn(x, x);
    const float xx_lo = __fmaf_rn(x, x, -xx);
    const float a = __fmul_rn(xx, half_log2e);
    const float a_lo = __fmaf_rn(xx_lo, half_log2e, __fmaf_rn(xx, half_log2e, -a));
    float g = __fmaf_rn(isp.hi, p, __fmul_rn(isp.lo, p));
    g = __fmaf_rn(g, __fmul_rn(a_lo, ln2), g);
    return __fmul_rn(ex2_approx(a), g);
}

// expm1(z) for the discount factor exp(-r t) - 1.  |z| <= 0.5: Taylor series
// to z^8 (truncation < 1.5e-8 relative); otherwise 2^(z log2 e) - 1 on the SFU.
__device__ __forceinline__ float expm1_disc(float z) {
    float p = __fmaf_rn(z, 1.0f / 40320.0f, 1.0f / 5040.0f);
    p = __fmaf_rn(z, p, 1.0f / 720.0f);
    p = __fmaf_rn(z, p, 1.0f / 120.0f);
    p = __fmaf_rn(z, p, 1.0f / 24.0f);
    p = __fmaf_rn(z, p, 1.0f / 6.0f);
    p = __fmaf_rn(z, p, 0.5f);
    p = __fmaf_rn(z, p, 1.0f);
    const float small = __fmul_rn(z, p);
    const float big = ex2_approx(__fmul_rn(z, (float)BSG_LOG2E)) - 1.0f;
    return (fabsf(z) <= 0.5f) ? small : big;
}

// Compensated FP32 price (production path).
//   d1 = ((r + v^2/2) t + ln(S/K)) / (v sqrt t), d2 = d1 - v sqrt t.
//   An error in d1 is shared by d2 and cancels to first order (S phi(d1) =
//   K e^{-rt} phi(d2)), so ln(S/K) and the division use the SFU.  v sqrt t
//   does not cancel (its error acts as a volatility error), so sqrt(t) gets
//   one Newton step.
//   N(d) = H(d) + sigma(d) Q(|d|) with H = [d >= 0], sigma = -1 if d >= 0
//   else +1; then call = S N1 - FV N2 and put = FV (1-N2) - S (1-N1) share
//   the Q terms and differ only in the H part, which is 0, S, FV or +-(S-FV).
//   FV = K (1 + m), m = expm1(-r t) with r t carried as float-float, so
//   S - FV = (S - K) - K m has no rounding of a ~K-sized FV.
__device__ __forceinline__ float price_fast(float s, float k, float r, float v,
                                            float t, int otype) {
    constexpr float ln2 = (float)BSG_LN2;
    const float rs = rsqrt_approx(t);
    float sq = __fmul_rn(t, rs);
    sq = __fmaf_rn(__fmaf_rn(-sq, sq, t), __fmul_rn(0.5f, rs), sq);
    // t = 0, inf, NaN or < 0: the IEEE-style answer of sqrt.approx
    sq = (t > 0.0f && t < 3.0e38f) ? sq : sqrt_approx(t);
    const float den = __fmul_rn(v, sq);
    const float lg = __fmul_rn(lg2_approx(__fmul_rn(s, rcp_approx(k))), ln2);
    const float num = __fmaf_rn(__fmaf_rn(__fmul_rn(0.5f, v), v, r), t, lg);
    const float d1 = __fmul_rn(num, rcp_approx(den));
    const float d2 = __fsub_rn(d1, den);

    const float q1 = tail_q(fabsf(d1));
    const float q2 = tail_q(fabsf(d2));

    const float rt = __fmul_rn(r, t);
    const float rt_lo = __fmaf_rn(r, t, -rt);
    float m = expm1_disc(-rt);
    m = __fmaf_rn(-rt_lo, 1.0f + m, m);
    const float fv = __fmaf_rn(k, m, k);
    const float s_fv = __fmaf_rn(-k, m, __fsub_rn(s, k));

    const bool h1 = d1 >= 0.0f;
    const bool h2 = d2 >= 0.0f;
    float h;
    if (otype == 0)
        h = h1 ? (h2 ? s_fv : s) : 0.0f;
    else
        h = h1 ? (h2 ? 0.0f : fv) : -s_fv;
    const float tq = __fmaf_rn(h1 ? -s : s, q1, h);
    const float price = __fmaf_rn(h2 ? fv : -fv, q2, tq);
    // NaN in d1 selects neither H branch consistently; make it propagate.
    return (d1 == d1) ? price : d1;
}

// ------------------------------------------------ two options per operation
// The compensated path for a pair of options at once: every FP32 add,
// multiply and fused multiply-add of price_fast becomes one packed f32x2
// operation (__fadd2_rn / __fmul2_rn / __ffma2_rn, sm_100+), whose result per
// component is that of the scalar operation.  SFU approximations, compares
// and selects stay per component.  The two components are therefore
// bit-identical to price_fast on each option, with about half the issued
// FP32 instructions.  One caveat, measured: the toolchain fuses a packed
// multiply into a packed add or subtract that is its only use, skipping the
// product's rounding.  No product here has that shape: each is an fma
// operand, is exact, or has several uses.
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }

__device__ __forceinline__ float2 tail_q2(float2 x) {
    constexpr FF c0 = split(BSG_C0);
    constexpr FF isp = split(BSG_INV_SQRT_2PI);
    constexpr float b0 = (float)(BSG_C1 + BSG_C2 + BSG_C3 + BSG_C4 + BSG_C5);
    constexpr float b1 = (float)(-(BSG_C2 + 2 * BSG_C3 + 3 * BSG_C4 + 4 * BSG_C5));
    constexpr float b2 = (float)(BSG_C3 + 3 * BSG_C4 + 6 * BSG_C5);
    constexpr float b3 = (float)(-(BSG_C4 + 4 * BSG_C5));
    constexpr float b4 = (float)BSG_C5;
    constexpr float half_log2e = (float)(-0.5 * BSG_LOG2E);
    constexpr float ln2 = (float)BSG_LN2;

    x.x = (x.x > 40.0f) ? 40.0f : x.x;
    x.y = (x.y > 40.0f) ? 40.0f : x.y;

    const float2 cx = mul2(f2(c0.hi), x);
    const float2 y = fma2(f2(c0.hi), x, f2(1.0f));
    const float2 y_lo = fma2(f2(c0.lo), x, fma2(f2(c0.hi), x, add2(f2(1.0f), neg2(y))));
    const float2 k0 = make_float2(rcp_approx(y.x), rcp_approx(y.y));
    const float2 k = fma2(k0, fma2(neg2(y), k0, f2(1.0f)), k0);
    const float2 res = fma2(neg2(y_lo), k, fma2(neg2(y), k, f2(1.0f)));
    const float2 k_lo = mul2(k, res);

    const float2 w = mul2(cx, k);
    float2 in = fma2(w, f2(b4), f2(b3));
    in = fma2(w, in, f2(b2));
    in = fma2(w, in, f2(b1));
    in = fma2(w, in, f2(b0));
    const float2 p = fma2(in, k_lo, mul2(in, k));

    const float2 xx = mul2(x, x);
    const float2 xx_lo = fma2(x, x, neg2(xx));
    const float2 a = mul2(xx, f2(half_log2e));
    const float2 a_lo = fma2(xx_lo, f2(half_log2e), fma2(xx, f2(half_log2e), neg2(a)));
    float2 g = fma2(f2(isp.hi), p, mul2(f2(isp.lo), p));
    g = fma2(g, mul2(a_lo, f2(ln2)), g);
    return mul2(make_float2(ex2_approx(a.x), ex2_approx(a.y)), g);
}

__device__ __forceinline__ float2 expm1_disc2(float2 z) {
    float2 p = fma2(z, f2(1.0f / 40320.0f), f2(1.0f / 5040.0f));
    p = fma2(z, p, f2(1.0f / 720.0f));
    p = fma2(z, p, f2(1.0f / 120.0f));
    p = fma2(z, p, f2(1.0f / 24.0f));
    p = fma2(z, p, f2(1.0f / 6.0f));
    p = fma2(z, p, f2(0.5f));
    p = fma2(z, p, f2(1.0f));
    const float2 small = mul2(z, p);
    const float2 zl = mul2(z, f2((float)BSG_LOG2E));
    const float2 big = add2(make_float2(ex2_approx(zl.x), ex2_approx(zl.y)), f2(-1.0f));
    return make_float2(fabsf(z.x) <= 0.5f ? small.x : big.x, fabsf(z.y) <= 0.5f ? small.y : big.y);
}

// price_fast's H part and signs for one option (see price_fast).
__device__ __forceinline__ void price_parts(float s, float fv, float s_fv, float d1, float d2,
                                            int otype, float& h, float& sq1, float& sq2) {
    const bool h1 = d1 >= 0.0f;
    const bool h2 = d2 >= 0.0f;
    if (otype == 0)
        h = h1 ? (h2 ? s_fv : s) : 0.0f;
    else
        h = h1 ? (h2 ? 0.0f : fv) : -s_fv;
    sq1 = h1 ? -s : s;
    sq2 = h2 ? fv : -fv;
}

__device__ __forceinline__ float2 price_fast2(float2 s, float2 k, float2 r, float2 v, float2 t,
                                              int ot0, int ot1) {
    constexpr float ln2 = (float)BSG_LN2;
    const float2 rs = make_float2(rsqrt_approx(t.x), rsqrt_approx(t.y));
    float2 sq = mul2(t, rs);
    sq = fma2(fma2(neg2(sq), sq, t), mul2(f2(0.5f), rs), sq);
    sq.x = (t.x > 0.0f && t.x < 3.0e38f) ? sq.x : sqrt_approx(t.x);
    sq.y = (t.y > 0.0f && t.y < 3.0e38f) ? sq.y : sqrt_approx(t.y);
    const float2 den = mul2(v, sq);
    const float2 q = mul2(s, make_float2(rcp_approx(k.x), rcp_approx(k.y)));
    const float2 lg = mul2(make_float2(lg2_approx(q.x), lg2_approx(q.y)), f2(ln2));
    const float2 num = fma2(fma2(mul2(f2(0.5f), v), v, r), t, lg);
    const float2 d1 = mul2(num, make_float2(rcp_approx(den.x), rcp_approx(den.y)));
    const float2 d2 = add2(d1, neg2(den));

    const float2 q1 = tail_q2(make_float2(fabsf(d1.x), fabsf(d1.y)));
    const float2 q2 = tail_q2(make_float2(fabsf(d2.x), fabsf(d2.y)));

    const float2 rt = mul2(r, t);
    const float2 rt_lo = fma2(r, t, neg2(rt));
    float2 m = expm1_disc2(neg2(rt));
    m = fma2(neg2(rt_lo), add2(f2(1.0f), m), m);
    const float2 fv = fma2(k, m, k);
    const float2 s_fv = fma2(neg2(k), m, add2(s, neg2(k)));

    float2 h, sq1, sq2;
    price_parts(s.x, fv.x, s_fv.x, d1.x, d2.x, ot0, h.x, sq1.x, sq2.x);
    price_parts(s.y, fv.y, s_fv.y, d1.y, d2.y, ot1, h.y, sq1.y, sq2.y);
    const float2 price = fma2(sq2, q2, fma2(sq1, q1, h));
    return make_float2((d1.x == d1.x) ? price.x : d1.x, (d1.y == d1.y) ? price.y : d1.y);
}

// ---------------------------------------------------- reference-order paths
// SFU flavour: blackscholes.c:126-258 step by step in FP32, every libm call
// and division replaced by its MUFU approximation, literals as floats.
__device__ __forceinline__ float cndf_sfu_ref(float x) {
    const bool neg = x < 0.0f;
    x = fabsf(x);
    const float e = ex2_approx(__fmul_rn(__fmul_rn(-0.5f, x), x) * (float)BSG_LOG2E);
    const float np = __fmul_rn(e, (float)BSG_INV_SQRT_2PI);
    float k = __fadd_rn(1.0f, __fmul_rn((float)BSG_C0, x));
    k = rcp_approx(k);
    const float k2 = __fmul_rn(k, k), k3 = __fmul_rn(k2, k);
    const float k4 = __fmul_rn(k3, k), k5 = __fmul_rn(k4, k);
    float l1 = __fmul_rn(k, (float)BSG_C1);
    float l2 = __fadd_rn(__fmul_rn(k2, (float)BSG_C2), __fmul_rn(k3, (float)BSG_C3));
    l2 = __fadd_rn(l2, __fmul_rn(k4, (float)BSG_C4));
    l2 = __fadd_rn(l2, __fmul_rn(k5, (float)BSG_C5));
    l1 = __fadd_rn(l2, l1);
    const float out = __fsub_rn(1.0f, __fmul_rn(l1, np));
    return neg ? __fsub_rn(1.0f, out) : out;
}

__device__ __forceinline__ float price_sfu_ref(float s, float k, float r, float v,
                                               float t, int otype) {
    const float sq = sqrt_approx(t);
    const float lg = __fmul_rn(lg2_approx(__fmul_rn(s, rcp_approx(k))), (float)BSG_LN2);
    float d1 = __fadd_rn(r, __fmul_rn(__fmul_rn(v, v), 0.5f));
    d1 = __fadd_rn(__fmul_rn(d1, t), lg);
    const float den = __fmul_rn(v, sq);
    d1 = __fmul_rn(d1, rcp_approx(den));
    const float d2 = __fsub_rn(d1, den);
    const float n1 = cndf_sfu_ref(d1), n2 = cndf_sfu_ref(d2);
    const float fv = __fmul_rn(k, ex2_approx(__fmul_rn(__fmul_rn(-r, t), (float)BSG_LOG2E)));
    if (otype == 0) return __fsub_rn(__fmul_rn(s, n1), __fmul_rn(fv, n2));
    return __fsub_rn(__fmul_rn(fv, __fsub_rn(1.0f, n2)), __fmul_rn(s, __fsub_rn(1.0f, n1)));
}

// float x double-literal product rounded to float, as the reference's
// `float = float * <double literal>` lines evaluate (to within the rare
// double-rounding case).  An infinite x gives c.hi * x, the double product's
// value (c.hi x + c.lo x would be inf - inf when c.lo has the other sign).
__device__ __forceinline__ float dmul_finite(float x, FF c) {
    return __fmaf_rn(c.hi, x, __fmul_rn(c.lo, x));
}
__device__ __forceinline__ float dmul(float x, FF c) {
    return isinf(x) ? __fmul_rn(c.hi, x) : dmul_finite(x, c);
}

__device__ __forceinline__ float cndf_libm_ref(float x) {
    constexpr FF c0 = split(BSG_C0), c1 = split(BSG_C1), c2 = split(BSG_C2);
    constexpr FF c3 = split(BSG_C3), c4 = split(BSG_C4), c5 = split(BSG_C5);
    constexpr FF isp = split(BSG_INV_SQRT_2PI);
    const bool neg = x < 0.0f;                                   // :146-150
    x = neg ? -x : x;
    // x = |d1| may be infinite (v sqrt(t) = 0); e and k = 1 / (1 + x c0)
    // are always finite (in [0, 1]), so only x c0 needs dmul's inf case
    const float e = bsg_cr::exp(__fmul_rn(__fmul_rn(-0.5f, x), x));  // :155
    const float np = dmul_finite(e, isp);                        // :157
    float k = dmul(x, c0);                                       // :159
    k = __fadd_rn(1.0f, k);                                      // :160
    k = __frcp_rn(k);  // :161, 1.0 / k in double rounded to float: the
                       // correctly rounded reciprocal
    const float k2 = __fmul_rn(k, k), k3 = __fmul_rn(k2, k);     // :162-165
    const float k4 = __fmul_rn(k3, k), k5 = __fmul_rn(k4, k);
    float l1 = dmul_finite(k, c1);                               // :167
    float l2 = dmul_finite(k2, c2);                              // :168
    float l3 = dmul_finite(k3, c3);                              // :169
    l2 = __fadd_rn(l2, l3);
    l3 = dmul_finite(k4, c4);
    l2 = __fadd_rn(l2, l3);
    l3 = dmul_finite(k5, c5);
    l2 = __fadd_rn(l2, l3);                                      // :174
    l1 = __fadd_rn(l2, l1);                                      // :176
    float out = __fmul_rn(l1, np);                               // :177
    out = __fsub_rn(1.0f, out);                                  // :178
    return neg ? __fsub_rn(1.0f, out) : out;                     // :182-184
}

__device__ __forceinline__ float price_libm_ref(float s, float k, float r, float v,
                                                float t, int otype) {
    const float sq = __fsqrt_rn(t);                              // :226
    const float lg = bsg_cr::log(__fdiv_rn(s, k));               // :228
    float pw = __fmul_rn(v, v);                                  // :233
    pw = __fmul_rn(pw, 0.5f);                                    // :234 (exact)
    float d1 = __fadd_rn(r, pw);                                 // :236
    d1 = __fmul_rn(d1, t);
    d1 = __fadd_rn(d1, lg);
    const float den = __fmul_rn(v, sq);                          // :240
    d1 = __fdiv_rn(d1, den);                                     // :241
    const float d2 = __fsub_rn(d1, den);                         // :242
    const float n1 = cndf_libm_ref(d1), n2 = cndf_libm_ref(d2);
    const float fv = __fmul_rn(k, bsg_cr::exp(__fmul_rn(-r, t)));  // :250
    if (otype == 0) return __fsub_rn(__fmul_rn(s, n1), __fmul_rn(fv, n2));
    const float nn1 = __fsub_rn(1.0f, n1), nn2 = __fsub_rn(1.0f, n2);
    return __fsub_rn(__fmul_rn(fv, nn2), __fmul_rn(s, nn1));     // :256
}

// Two options at a time: the operations of cndf_libm_ref / price_libm_ref
// and of bsg_cr::exp / bsg_cr::log, each as one packed f32x2 operation
// where the scalar code has a float operation (componentwise the same
// rounding: the same bits), per lane where it has a division, a square
// root, integer work or a table load -- and per lane where the reference
// rounds a product and then adds it: the toolchain fuses an f32x2 multiply
// into the f32x2 add or subtract that is its only use (even from inline
// PTX mul.rn.f32x2 / add.rn.f32x2, and under -fmad=false), which would skip
// that rounding.
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return add2(a, neg2(b)); }
struct FF2 { float2 hi, lo; };
__device__ __forceinline__ FF2 two_sum2(float2 a, float2 b) {
    const float2 s = add2(a, b);
    const float2 bb = sub2(s, a);
    return {s, add2(sub2(a, sub2(s, bb)), sub2(b, bb))};
}
__device__ __forceinline__ FF2 fast_two_sum2(float2 a, float2 b) {
    const float2 s = add2(a, b);
    return {s, sub2(b, sub2(s, a))};
}
__device__ __forceinline__ FF2 two_prod2(float2 a, float2 b) {
    const float2 p = mul2(a, b);
    return {p, fma2(a, b, neg2(p))};
}
__device__ __forceinline__ bool cr_exp_in_range(float x) { return x >= -87.0f && x <= 88.5f; }
__device__ __forceinline__ bool cr_log_in_range(float x) {
    return x >= 1.17549435e-38f && x <= 3.40282347e38f;
}

// A lane whose argument is outside bsg_cr::exp's domain takes the platform's
// expf, as bsg_cr::exp does; the packed evaluation runs on 0 in its place.
__device__ __forceinline__ float2 cr_exp2(float2 xin) {
    const bool in0 = cr_exp_in_range(xin.x), in1 = cr_exp_in_range(xin.y);
    const float2 x = make_float2(in0 ? xin.x : 0.0f, in1 ? xin.y : 0.0f);
    const float2 sh = fma2(x, f2(BSG_CR_INV_L), f2(bsg_cr::kShifter));
    const float2 nf = sub2(sh, f2(bsg_cr::kShifter));
    const int n0 = (int)(__float_as_uint(sh.x) - bsg_cr::kShifterBits);
    const int n1 = (int)(__float_as_uint(sh.y) - bsg_cr::kShifterBits);
    const float2 r1 = fma2(neg2(nf), f2(BSG_CR_L1), x);
    const FF2 p = two_prod2(nf, f2(BSG_CR_L2));
    const FF2 rs = two_sum2(r1, neg2(p.hi));
    const float2 rh = rs.hi;
    const float2 rl = fma2(neg2(nf), f2(BSG_CR_L3), sub2(rs.lo, p.lo));
    const FF2 s2 = two_prod2(rh, rh);
    float2 c = fma2(rh, f2(1.0f / 120.0f), f2(1.0f / 24.0f));
    c = fma2(rh, c, f2(1.0f / 6.0f));
    c = mul2(rh, c);
    const FF2 q = fast_two_sum2(rh, mul2(s2.hi, f2(0.5f)));
    const float2 ql =
        add2(q.lo, add2(rl, fma2(s2.lo, f2(0.5f), fma2(rh, rl, mul2(s2.hi, c)))));
    const bsg_cr::F2 t0 = bsg_cr::exp_tab(n0 & 31), t1 = bsg_cr::exp_tab(n1 & 31);
    const float2 thi = make_float2(t0.hi, t1.hi), tlo = make_float2(t0.lo, t1.lo);
    const FF2 tq = two_prod2(thi, q.hi);
    const FF2 sm = fast_two_sum2(thi, tq.hi);
    const float2 lo = add2(sm.lo, add2(tq.lo, add2(tlo, fma2(thi, ql, mul2(tlo, q.hi)))));
    const float2 y = add2(sm.hi, lo);
    float2 e = mul2(y, make_float2(__uint_as_float((uint32_t)((n0 >> 5) + 127) << 23),
                                   __uint_as_float((uint32_t)((n1 >> 5) + 127) << 23)));
    if (!in0) e.x = bsg_cr::fallback_exp(xin.x);
    if (!in1) e.y = bsg_cr::fallback_exp(xin.y);
    return e;
}

__device__ __forceinline__ float2 cr_log2(float2 x) {
    if (!(cr_log_in_range(x.x) && cr_log_in_range(x.y)))
        return make_float2(bsg_cr::log(x.x), bsg_cr::log(x.y));
    const uint32_t u0 = __float_as_uint(x.x), u1 = __float_as_uint(x.y);
    const uint32_t i0 = (u0 >> 15) & 0xFFu, i1 = (u1 >> 15) & 0xFFu;
    const int e0 = (int)(u0 >> 23) - 127 + (int)(i0 >> 7);
    const int e1 = (int)(u1 >> 23) - 127 + (int)(i1 >> 7);
    const float2 m = make_float2(
        __uint_as_float((u0 & 0x7FFFFFu) | (i0 >= 128 ? 0x3F000000u : 0x3F800000u)),
        __uint_as_float((u1 & 0x7FFFFFu) | (i1 >= 128 ? 0x3F000000u : 0x3F800000u)));
    const bsg_cr::LogEntry g0 = bsg_cr::log_tab((int)i0), g1 = bsg_cr::log_tab((int)i1);
    const float2 r = fma2(m, make_float2(g0.c, g1.c), f2(-1.0f));
    const FF2 s2 = two_prod2(r, r);
    float2 c = fma2(r, f2(0.2f), f2(-0.25f));
    c = fma2(r, c, f2(1.0f / 3.0f));
    c = mul2(mul2(s2.hi, r), c);
    const FF2 a = fast_two_sum2(r, mul2(s2.hi, f2(-0.5f)));
    const float2 alo = add2(a.lo, fma2(s2.lo, f2(-0.5f), c));
    const float2 ef = sub2(make_float2(__uint_as_float(bsg_cr::kShifterBits + (uint32_t)e0),
                                       __uint_as_float(bsg_cr::kShifterBits + (uint32_t)e1)),
                           f2(bsg_cr::kShifter));
    const FF2 em = two_prod2(ef, f2(BSG_CR_LN2M));
    const FF2 s1 = two_sum2(mul2(ef, f2(BSG_CR_LN2H)), make_float2(g0.hi, g1.hi));
    const FF2 s2s = two_sum2(s1.hi, a.hi);
    const FF2 s3 = two_sum2(s2s.hi, em.hi);
    const float2 lo = add2(add2(add2(s1.lo, s2s.lo), s3.lo),
                           add2(add2(make_float2(g0.lo, g1.lo), alo),
                                fma2(ef, f2(BSG_CR_LN2L), em.lo)));
    return add2(s3.hi, lo);
}

__device__ __forceinline__ float2 dmul_finite2(float2 x, FF c) {
    return fma2(f2(c.hi), x, mul2(f2(c.lo), x));
}

__device__ __forceinline__ float2 cndf_libm_ref2(float2 xin) {
    constexpr FF c0 = split(BSG_C0), c1 = split(BSG_C1), c2 = split(BSG_C2);
    constexpr FF c3 = split(BSG_C3), c4 = split(BSG_C4), c5 = split(BSG_C5);
    constexpr FF isp = split(BSG_INV_SQRT_2PI);
    const bool neg0 = xin.x < 0.0f, neg1 = xin.y < 0.0f;
    const float2 x = make_float2(neg0 ? -xin.x : xin.x, neg1 ? -xin.y : xin.y);
    const float2 e = cr_exp2(mul2(mul2(f2(-0.5f), x), x));
    const float2 np = dmul_finite2(e, isp);
    float2 k = make_float2(dmul(x.x, c0), dmul(x.y, c0));
    k = add2(f2(1.0f), k);
    k = make_float2(__frcp_rn(k.x), __frcp_rn(k.y));
    const float2 k2 = mul2(k, k), k3 = mul2(k2, k);
    const float2 k4 = mul2(k3, k), k5 = mul2(k4, k);
    float2 l1 = dmul_finite2(k, c1);
    float2 l2 = dmul_finite2(k2, c2);
    float2 l3 = dmul_finite2(k3, c3);
    l2 = add2(l2, l3);
    l3 = dmul_finite2(k4, c4);
    l2 = add2(l2, l3);
    l3 = dmul_finite2(k5, c5);
    l2 = add2(l2, l3);
    l1 = add2(l2, l1);
    const float2 out = make_float2(__fsub_rn(1.0f, __fmul_rn(l1.x, np.x)),
                                   __fsub_rn(1.0f, __fmul_rn(l1.y, np.y)));
    const float2 refl = sub2(f2(1.0f), out);
    return make_float2(neg0 ? refl.x : out.x, neg1 ? refl.y : out.y);
}

__device__ __forceinline__ float2 price_libm_ref2(float2 s, float2 k, float2 r, float2 v,
                                                  float2 t, int ot0, int ot1) {
    const float2 sq = make_float2(__fsqrt_rn(t.x), __fsqrt_rn(t.y));
    const float2 lg = cr_log2(make_float2(__fdiv_rn(s.x, k.x), __fdiv_rn(s.y, k.y)));
    float2 pw = mul2(v, v);
    pw = mul2(pw, f2(0.5f));
    float2 d1 = add2(r, pw);
    d1 = make_float2(__fadd_rn(__fmul_rn(d1.x, t.x), lg.x), __fadd_rn(__fmul_rn(d1.y, t.y), lg.y));
    const float2 den = mul2(v, sq);
    d1 = make_float2(__fdiv_rn(d1.x, den.x), __fdiv_rn(d1.y, den.y));
    const float2 d2 = sub2(d1, den);
    const float2 n1 = cndf_libm_ref2(d1), n2 = cndf_libm_ref2(d2);
    const float2 fv = mul2(k, cr_exp2(mul2(neg2(r), t)));
    const float2 nn1 = sub2(f2(1.0f), n1), nn2 = sub2(f2(1.0f), n2);
    const float p0 = ot0 == 0 ? __fsub_rn(__fmul_rn(s.x, n1.x), __fmul_rn(fv.x, n2.x))
                              : __fsub_rn(__fmul_rn(fv.x, nn2.x), __fmul_rn(s.x, nn1.x));
    const float p1 = ot1 == 0 ? __fsub_rn(__fmul_rn(s.y, n1.y), __fmul_rn(fv.y, n2.y))
                              : __fsub_rn(__fmul_rn(fv.y, nn2.y), __fmul_rn(s.y, nn1.y));
    return make_float2(p0, p1);
}

// ------------------------------------------------------------------- FP64
// The same formula in double, operation for operation as the reference's
// NCO = 2 SIMD build evaluates it (blackscholes.simd.c:134-298), with
// explicitly rounded operations (no fused multiply-adds): only CUDA's double
// exp/log can differ from the host libm's, by an ulp.
__device__ __forceinline__ double cndf_fp64(double x) {
    const bool neg = x < 0.0;
    x = neg ? -x : x;
    const double np = __dmul_rn(exp(__dmul_rn(__dmul_rn(-0.5, x), x)), BSG_INV_SQRT_2PI);
    const double k = __ddiv_rn(1.0, __dadd_rn(1.0, __dmul_rn(BSG_C0, x)));
    const double k2 = __dmul_rn(k, k), k3 = __dmul_rn(k2, k);
    const double k4 = __dmul_rn(k3, k), k5 = __dmul_rn(k4, k);
    double l2 = __dadd_rn(__dmul_rn(k2, BSG_C2), __dmul_rn(k3, BSG_C3));
    l2 = __dadd_rn(l2, __dmul_rn(k4, BSG_C4));
    l2 = __dadd_rn(l2, __dmul_rn(k5, BSG_C5));
    const double l1 = __dadd_rn(l2, __dmul_rn(k, BSG_C1));
    const double out = __dsub_rn(1.0, __dmul_rn(l1, np));
    return neg ? __dsub_rn(1.0, out) : out;
}

__device__ __forceinline__ double d1_fp64(double s, double k, double r, double v, double t) {
    const double num = __dadd_rn(__dmul_rn(__dadd_rn(r, __dmul_rn(__dmul_rn(v, v), 0.5)), t),
                                 log(__ddiv_rn(s, k)));
    return __ddiv_rn(num, __dmul_rn(v, __dsqrt_rn(t)));
}

__device__ __forceinline__ double price_fp64(double s, double k, double r, double v,
                                             double t, int otype) {
    const double den = __dmul_rn(v, __dsqrt_rn(t));
    const double num = __dadd_rn(__dmul_rn(__dadd_rn(r, __dmul_rn(__dmul_rn(v, v), 0.5)), t),
                                 log(__ddiv_rn(s, k)));
    const double d1 = __ddiv_rn(num, den);
    const double d2 = __dsub_rn(d1, den);
    const double n1 = cndf_fp64(d1), n2 = cndf_fp64(d2);
    const double fv = __dmul_rn(k, exp(__dmul_rn(-r, t)));
    if (otype == 0) return __dsub_rn(__dmul_rn(s, n1), __dmul_rn(fv, n2));
    return __dsub_rn(__dmul_rn(fv, __dsub_rn(1.0, n2)), __dmul_rn(s, __dsub_rn(1.0, n1)));
}

template <int M>
__device__ __forceinline__ float price(float s, float k, float r, float v, float t, int ot) {
    if constexpr (M == MODE_FAST) return price_fast(s, k, r, v, t, ot);
    else if constexpr (M == MODE_SFU_REF) return price_sfu_ref(s, k, r, v, t, ot);
    else return price_libm_ref(s, k, r, v, t, ot);
}

// Four consecutive options (the FAST path two at a time in f32x2 operations;
// the same bits as four calls of price<M>).
template <int M>
__device__ __forceinline__ float4 price4(float4 s, float4 k, float4 r, float4 v, float4 t,
                                         int4 ot) {
    if constexpr (M == MODE_FAST) {
        const float2 a = price_fast2(make_float2(s.x, s.y), make_float2(k.x, k.y),
                                     make_float2(r.x, r.y), make_float2(v.x, v.y),
                                     make_float2(t.x, t.y), ot.x, ot.y);
        const float2 b = price_fast2(make_float2(s.z, s.w), make_float2(k.z, k.w),
                                     make_float2(r.z, r.w), make_float2(v.z, v.w),
                                     make_float2(t.z, t.w), ot.z, ot.w);
        return make_float4(a.x, a.y, b.x, b.y);
    } else if constexpr (M == MODE_LIBM_REF) {
        const float2 a = price_libm_ref2(make_float2(s.x, s.y), make_float2(k.x, k.y),
                                         make_float2(r.x, r.y), make_float2(v.x, v.y),
                                         make_float2(t.x, t.y), ot.x, ot.y);
        const float2 b = price_libm_ref2(make_float2(s.z, s.w), make_float2(k.z, k.w),
                                         make_float2(r.z, r.w), make_float2(v.z, v.w),
                                         make_float2(t.z, t.w), ot.z, ot.w);
        return make_float4(a.x, a.y, b.x, b.y);
    } else {
        return make_float4(price<M>(s.x, k.x, r.x, v.x, t.x, ot.x),
                           price<M>(s.y, k.y, r.y, v.y, t.y, ot.y),
                           price<M>(s.z, k.z, r.z, v.z, t.z, ot.z),
                           price<M>(s.w, k.w, r.w, v.w, t.w, ot.w));
    }
}

}  // namespace bsg
