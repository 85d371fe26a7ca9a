/*
 * swpt_oracle.h -- CPU oracle for the swaption Monte Carlo (TEST
 * INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's CPU
 * legs may load it; libbsgpu.so never does).
 *
 * P3ARSEC's swaptions application prices each swaption with
 * HJM_Swaption_Blocking (parsec-ff/pkgs/apps/swaptions/src/
 * HJM_Swaption_Blocking.cpp:19-223) inside a FastFlow ParallelFor over the
 * swaptions (HJM_Securities.cpp:312-323).  The reference tree holds that
 * driver but not the model core it calls (HJM_Yield_to_Forward, HJM_Drifts,
 * HJM_SimPath_Forward_Blocking, Discount_Factors_Blocking, RanUnif,
 * CumNormalInv: nr_routines.h / HJM.h are not in the tree), so parity with
 * the reference is UNPINNED.  This file restates:
 *
 *  - the driver's arithmetic as the reference writes it: the strike's
 *    continuous-compounding conversion, the index rounding, the swap
 *    payment vector, the fixed-leg value, the floored payoff, its discount
 *    and the mean / standard-error accumulation (HJM_Swaption_Blocking.cpp:
 *    48-62, 116-140, 165-214);
 *  - the model core from its published form: the discrete-time HJM model of
 *    Heath, Jarrow and Morton (Econometrica 60(1), 1992) in the
 *    time-to-maturity (Musiela) parameterisation with the drift that makes
 *    discounted bond prices exact martingales of the discretised model:
 *    for a Gaussian step, E[exp(-h sum_j df_j)] = 1 for every maturity
 *    forces mu[m] = (h/2) sum_k (S_k(m)^2 - S_k(m-1)^2), with S_k(m) the
 *    sum of factor k's vols over maturities 0..m (Glasserman, Monte Carlo
 *    Methods in Financial Engineering, 2003, section 3.6.2, states the same
 *    condition);
 *  - normal variates from a counter-based generator (Philox4x32-10, Salmon,
 *    Moraes, Dror and Shaw, SC'11) through the Box-Muller transform, so that
 *    every trial's variates depend only on (seed, trial, index) and the GPU
 *    kernel can draw the same ones in any order.  The reference's own RanUnif
 *    / CumNormalInv stream is not reproduced (not in the tree).
 *
 * Everything is double precision, as the reference's FTYPE.
 */
#ifndef SWPT_ORACLE_H
#define SWPT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One swaption, the reference's parm fields (HJM_Securities.cpp:276-296). */
typedef struct swo_swaption {
    double strike, compounding, maturity, tenor, payment_interval, years;
    int n_steps;            /* iN */
    int n_factors;          /* iFactors */
    const double* yield;    /* n_steps */
    const double* factors;  /* n_factors x (n_steps - 1), row-major */
    uint64_t seed;
} swo_swaption;

/* Philox4x32-10 of counter c[4] under key k[2] into out[4]. */
void swo_philox4x32_10(const uint32_t c[4], const uint32_t k[2], uint32_t out[4]);

/* Normal variates 2j and 2j + 1 of one trial: Box-Muller of the two 52-bit
 * uniforms that Philox draws for counter (trial, j). */
void swo_normal_pair(uint64_t seed, uint64_t trial, uint32_t j, double z[2]);

/* Forward curve f[0..n) from the yield curve: f[0] = y[0], f[i] = (i+1) y[i]
 * - i y[i-1] (continuously compounded yields are running means of the
 * forwards). */
void swo_yield_to_forward(int n, const double* yield, double* fwd);

/* Risk-neutral drift mu[0..n-1) of the forward with time to maturity
 * m + 1 steps, factor vols v[k][m], step h. */
void swo_drift(int n, int nf, const double* v, double h, double* mu);

/* Prices one swaption with `trials` Monte Carlo paths, simulating the whole
 * HJM path matrix as the reference does.  out[0] = mean discounted payoff,
 * out[1] = its standard error.  flags bit 0: drop the floor (payoff V - 1
 * instead of max(V - 1, 0); the test of the drift).  Returns 1 on success,
 * 0 on arguments the reference would index out of bounds with. */
int swo_price(const swo_swaption* sw, uint64_t trials, unsigned flags, double out[2]);

/* Every swaption on nthreads threads, a static partition over swaptions
 * (the reference's ParallelFor with PARFOR_STATIC(0)).  Returns wall
 * seconds, or a negative value on an error. */
double swo_price_all(const swo_swaption* sw, int n, uint64_t trials, int nthreads,
                     double* price, double* stderr_out);

#ifdef __cplusplus
}
#endif
#endif /* SWPT_ORACLE_H */
