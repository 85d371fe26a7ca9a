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
//   price_libm_ref  the reference's operation order with CUDA's accurate
//                   expf/logf, IEEE division and square root, and the
//                   reference's double-literal products emulated in FP32.
//   price_fp64      the same formula in double (validation oracle).
//
// Every function here is branch-free per option apart from selects, and uses
// only explicit intrinsics (__fmaf_rn etc.) in the FP32 paths, so the result
// for an option never depends on where or with what it is priced.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

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
// double-rounding case).
__device__ __forceinline__ float dmul(float x, FF c) {
    return __fmaf_rn(c.hi, x, __fmul_rn(c.lo, x));
}

__device__ __forceinline__ float cndf_libm_ref(float x) {
    constexpr FF c0 = split(BSG_C0), c1 = split(BSG_C1), c2 = split(BSG_C2);
    constexpr FF c3 = split(BSG_C3), c4 = split(BSG_C4), c5 = split(BSG_C5);
    constexpr FF isp = split(BSG_INV_SQRT_2PI);
    const bool neg = x < 0.0f;                                   // :146-150
    x = neg ? -x : x;
    const float e = expf(__fmul_rn(__fmul_rn(-0.5f, x), x));     // :155
    const float np = dmul(e, isp);                               // :157
    float k = dmul(x, c0);                                       // :159
    k = __fadd_rn(1.0f, k);                                      // :160
    k = __fdiv_rn(1.0f, k);                                      // :161
    const float k2 = __fmul_rn(k, k), k3 = __fmul_rn(k2, k);     // :162-165
    const float k4 = __fmul_rn(k3, k), k5 = __fmul_rn(k4, k);
    float l1 = dmul(k, c1);                                      // :167
    float l2 = dmul(k2, c2);                                     // :168
    float l3 = dmul(k3, c3);                                     // :169
    l2 = __fadd_rn(l2, l3);
    l3 = dmul(k4, c4);
    l2 = __fadd_rn(l2, l3);
    l3 = dmul(k5, c5);
    l2 = __fadd_rn(l2, l3);                                      // :174
    l1 = __fadd_rn(l2, l1);                                      // :176
    float out = __fmul_rn(l1, np);                               // :177
    out = __fsub_rn(1.0f, out);                                  // :178
    return neg ? __fsub_rn(1.0f, out) : out;                     // :182-184
}

__device__ __forceinline__ float price_libm_ref(float s, float k, float r, float v,
                                                float t, int otype) {
    const float sq = __fsqrt_rn(t);                              // :226
    const float lg = logf(__fdiv_rn(s, k));                      // :228
    float pw = __fmul_rn(v, v);                                  // :233
    pw = __fmul_rn(pw, 0.5f);                                    // :234 (exact)
    float d1 = __fadd_rn(r, pw);                                 // :236
    d1 = __fmul_rn(d1, t);
    d1 = __fadd_rn(d1, lg);
    const float den = __fmul_rn(v, sq);                          // :240
    d1 = __fdiv_rn(d1, den);                                     // :241
    const float d2 = __fsub_rn(d1, den);                         // :242
    const float n1 = cndf_libm_ref(d1), n2 = cndf_libm_ref(d2);
    const float fv = __fmul_rn(k, expf(__fmul_rn(-r, t)));       // :250
    if (otype == 0) return __fsub_rn(__fmul_rn(s, n1), __fmul_rn(fv, n2));
    const float nn1 = __fsub_rn(1.0f, n1), nn2 = __fsub_rn(1.0f, n2);
    return __fsub_rn(__fmul_rn(fv, nn2), __fmul_rn(s, nn1));     // :256
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

}  // namespace bsg
