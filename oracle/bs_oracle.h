/*
 * bs_oracle.h -- CPU oracle for the Black-Scholes map (TEST INFRASTRUCTURE ONLY).
 *
 * This library is the checker, never the product: only tests/, the smoke
 * check in __graft_entry__.py and the cpu_baseline / reference legs of
 * bench.py may load it.  The GPU library (libbsgpu.so) never links it and
 * has no CPU fallback.
 *
 * Two restatements of the reference algorithm
 * (parsec-ff/pkgs/apps/blackscholes/src/blackscholes.c):
 *
 *   bso_*_ref   FP32 storage with the reference's double-precision constants,
 *               operation for operation as the reference compiled as C++
 *               evaluates it (float overloads expf/logf/sqrtf; every
 *               float-times-double literal is a double op rounded to float
 *               on assignment).  Built with -ffp-contract=off this is
 *               bit-identical to the reference on the same inputs (pinned
 *               against the compiled reference by tests/golden).
 *   bso_*_fp64  The same CNDF polynomial and pricing formula evaluated in
 *               double throughout on the float32 inputs: the accuracy oracle.
 */
#ifndef BS_ORACLE_H
#define BS_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* blackscholes.c:126-184 */
float  bso_cndf_ref(float x);
/* blackscholes.c:190-258 (timet is unused by the reference, so it is absent) */
float  bso_price_ref(float s, float k, float r, float v, float t, int otype);
/* The same operations with exp/log correctly rounded to float in place of
 * glibc's expf/logf (the rounding the GPU's reference-order mode targets). */
float  bso_price_ref_cr(float s, float k, float r, float v, float t, int otype);

double bso_cndf_fp64(double x);
double bso_price_fp64(double s, double k, double r, double v, double t, int otype);
/* d1 of the FP64 formula (used to bucket errors by CNDF tail) */
double bso_d1_fp64(double s, double k, double r, double v, double t);

/* Batch forms over SoA arrays: prices[i] = f(s[i], ..., otype[i]). */
void bso_price_ref_soa(size_t n, const float* s, const float* k, const float* r,
                       const float* v, const float* t, const int32_t* otype,
                       float* prices);
void bso_price_ref_cr_soa(size_t n, const float* s, const float* k, const float* r,
                          const float* v, const float* t, const int32_t* otype,
                          float* prices);
void bso_price_fp64_soa(size_t n, const float* s, const float* k, const float* r,
                        const float* v, const float* t, const int32_t* otype,
                        double* prices);

/* The FP64 formula over double inputs (the SIMD variant's NCO = 2 storage). */
void bso_price_fp64_soa_d(size_t n, const double* s, const double* k, const double* r,
                          const double* v, const double* t, const int32_t* otype,
                          double* prices);

/* Static block partition of [0, n) over nw workers, as FastFlow's default
 * static scheduling does (ff/parallel_for_internals.hpp:498-519): nw
 * contiguous blocks of floor(n/nw) options, the first n % nw blocks one
 * option larger.  Writes block w's [begin, end) to begin[w], end[w]. */
void bso_static_partition(int64_t n, int nw, int64_t* begin, int64_t* end);

/* The reference's FastFlow map driver restated (blackscholes.c:315-348):
 * num_runs passes, each a static-partition parallel-for over nthreads
 * workers with a join between passes.  Returns wall seconds of the ROI
 * (all passes), or a negative value on a thread error. */
double bso_bs_map(int nthreads, int num_runs, size_t n, const float* s,
                  const float* k, const float* r, const float* v,
                  const float* t, const int32_t* otype, float* prices);

/* The reference's sequential text I/O (blackscholes.c:695-767, 923-947):
 * the baseline the parallel I/O of libbsgpu.so is measured against. */
long bso_read_parsec_fscanf(const char* path, size_t cap, float* s, float* k,
                            float* r, float* v, float* t, int32_t* otype,
                            float* dgrefval);
int bso_write_prices_fprintf(const char* path, const float* prices, size_t n);

#ifdef __cplusplus
}
#endif
#endif /* BS_ORACLE_H */
