/*
 * bs_oracle.c -- CPU oracle for the Black-Scholes map (TEST INFRASTRUCTURE ONLY).
 *
 * The checker for the GPU library, never part of it.  Compile with
 * -ffp-contract=off: the reference's arithmetic has no fused multiply-adds
 * on x86-64, and the FP32 restatement must round exactly where it rounds
 * (gcc contracts a*b+c by default on aarch64).
 */
#define _GNU_SOURCE
#include "bs_oracle.h"

#include <math.h>
#include <stdint.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <time.h>

/* blackscholes.c:124 -- a double literal; products with it are double ops */
#define BSO_INV_SQRT_2PI 0.39894228040143270286

/*
 * CNDF, blackscholes.c:126-184.  Abramowitz & Stegun 26.2.17.
 * Every variable of the reference is a float; every literal is a double, so
 * each `float = float op double` line below is a double operation rounded to
 * float on assignment, as in the reference.  exp() of a float argument in
 * the reference (a C++ translation unit) resolves to expf.
 */
/* The reference's expf/logf (glibc), or, with cr set, exp/log correctly
 * rounded to float (through double: exact to within double rounding) -- the
 * rounding the GPU's reference-order mode targets. */
static float ref_exp(float x, int cr) { return cr ? (float)exp((double)x) : expf(x); }
static float ref_log(float x, int cr) { return cr ? (float)log((double)x) : logf(x); }

static float cndf_ref(float x, int cr)
{
    int sign = 0;
    if (x < 0.0) {                               /* :146-150 */
        x = -x;
        sign = 1;
    }
    const float xin = x;
    const float e = ref_exp(-0.5f * x * x, cr);  /* :155 float product, expf */
    const float nprime = e * BSO_INV_SQRT_2PI;   /* :157 double, rounded */

    float k = 0.2316419 * xin;                   /* :159-161 three roundings */
    k = 1.0 + k;
    k = 1.0 / k;
    const float k2 = k * k;                      /* :162-165 float */
    const float k3 = k2 * k;
    const float k4 = k3 * k;
    const float k5 = k4 * k;

    float l1 = k * 0.319381530;                  /* :167 */
    float l2 = k2 * (-0.356563782);              /* :168 */
    float l3 = k3 * 1.781477937;                 /* :169 */
    l2 = l2 + l3;                                /* :170 */
    l3 = k4 * (-1.821255978);                    /* :171 */
    l2 = l2 + l3;                                /* :172 */
    l3 = k5 * 1.330274429;                       /* :173 */
    l2 = l2 + l3;                                /* :174 */

    l1 = l2 + l1;                                /* :176 */
    float out = l1 * nprime;                     /* :177 */
    out = 1.0 - out;                             /* :178 double, rounded */
    if (sign) out = 1.0 - out;                   /* :182-184 */
    return out;
}

float bso_cndf_ref(float x) { return cndf_ref(x, 0); }

/* BlkSchlsEqEuroNoDiv, blackscholes.c:190-258 */
static float price_ref(float s, float k, float r, float v, float t, int otype, int cr)
{
    const float sqrt_t = sqrtf(t);               /* :226 */
    const float lg = ref_log(s / k, cr);         /* :228 */
    float power = v * v;                         /* :233 */
    power = power * 0.5;                         /* :234 double, rounded */
    float d1 = r + power;                        /* :236-238 */
    d1 = d1 * t;
    d1 = d1 + lg;
    const float den = v * sqrt_t;                /* :240 */
    d1 = d1 / den;                               /* :241 */
    const float d2 = d1 - den;                   /* :242 */

    const float n1 = cndf_ref(d1, cr);           /* :247-248 */
    const float n2 = cndf_ref(d2, cr);

    const float fv = k * ref_exp(-(r) * (t), cr);  /* :250 */
    float price;
    if (otype == 0) {
        price = (s * n1) - (fv * n2);            /* :252 */
    } else {
        const float nn1 = 1.0 - n1;              /* :254-255 double, rounded */
        const float nn2 = 1.0 - n2;
        price = (fv * nn2) - (s * nn1);          /* :256 */
    }
    return price;
}

float bso_price_ref(float s, float k, float r, float v, float t, int otype)
{
    return price_ref(s, k, r, v, t, otype, 0);
}

float bso_price_ref_cr(float s, float k, float r, float v, float t, int otype)
{
    return price_ref(s, k, r, v, t, otype, 1);
}

/* The same polynomial and summation order in double throughout. */
double bso_cndf_fp64(double x)
{
    int sign = 0;
    if (x < 0.0) {
        x = -x;
        sign = 1;
    }
    const double nprime = exp(-0.5 * x * x) * BSO_INV_SQRT_2PI;
    const double k = 1.0 / (1.0 + 0.2316419 * x);
    const double k2 = k * k, k3 = k2 * k, k4 = k3 * k, k5 = k4 * k;
    double l2 = k2 * (-0.356563782) + k3 * 1.781477937;
    l2 = l2 + k4 * (-1.821255978);
    l2 = l2 + k5 * 1.330274429;
    const double l1 = l2 + k * 0.319381530;
    double out = 1.0 - l1 * nprime;
    if (sign) out = 1.0 - out;
    return out;
}

double bso_d1_fp64(double s, double k, double r, double v, double t)
{
    return ((r + v * v * 0.5) * t + log(s / k)) / (v * sqrt(t));
}

double bso_price_fp64(double s, double k, double r, double v, double t, int otype)
{
    const double den = v * sqrt(t);
    const double d1 = ((r + v * v * 0.5) * t + log(s / k)) / den;
    const double d2 = d1 - den;
    const double n1 = bso_cndf_fp64(d1);
    const double n2 = bso_cndf_fp64(d2);
    const double fv = k * exp(-r * t);
    if (otype == 0) return s * n1 - fv * n2;
    return fv * (1.0 - n2) - s * (1.0 - n1);
}

void bso_price_ref_soa(size_t n, const float* s, const float* k, const float* r,
                       const float* v, const float* t, const int32_t* otype,
                       float* prices)
{
    for (size_t i = 0; i < n; ++i)
        prices[i] = bso_price_ref(s[i], k[i], r[i], v[i], t[i], otype[i]);
}

void bso_price_ref_cr_soa(size_t n, const float* s, const float* k, const float* r,
                          const float* v, const float* t, const int32_t* otype,
                          float* prices)
{
    for (size_t i = 0; i < n; ++i)
        prices[i] = bso_price_ref_cr(s[i], k[i], r[i], v[i], t[i], otype[i]);
}

void bso_price_fp64_soa(size_t n, const float* s, const float* k, const float* r,
                        const float* v, const float* t, const int32_t* otype,
                        double* prices)
{
    for (size_t i = 0; i < n; ++i)
        prices[i] = bso_price_fp64(s[i], k[i], r[i], v[i], t[i], otype[i]);
}

/* ff/parallel_for_internals.hpp:498-519 (default static scheduling, step 1) */
void bso_static_partition(int64_t n, int nw, int64_t* begin, int64_t* end)
{
    const int64_t chunk = n / nw;
    const int64_t rem = n % nw;
    int64_t start = 0;
    for (int w = 0; w < nw; ++w) {
        int64_t e = start + chunk + (w < rem ? 1 : 0);
        if (e > n) e = n;
        begin[w] = start;
        end[w] = e;
        start = e;
    }
}

/* ---- threaded map driver: num_runs passes, join between passes ---------- */

/* One pass is released by bumping `gen` (ff_loadbalancer::thawWorkers) and
 * joined when `ndone` reaches the worker count (wait_freezing). */
typedef struct {
    pthread_mutex_t mu;
    pthread_cond_t go, fin;
    int gen, ndone, quit;
} bso_gate;

typedef struct {
    bso_gate* g;
    int64_t begin, end;
    const float *s, *k, *r, *v, *t;
    const int32_t* otype;
    float* prices;
} bso_worker;

static void* bso_worker_main(void* arg)
{
    bso_worker* w = (bso_worker*)arg;
    bso_gate* g = w->g;
    int seen = 0;
    for (;;) {
        pthread_mutex_lock(&g->mu);
        while (g->gen == seen && !g->quit) pthread_cond_wait(&g->go, &g->mu);
        const int quit = g->quit;
        seen = g->gen;
        pthread_mutex_unlock(&g->mu);
        if (quit) return NULL;
        for (int64_t i = w->begin; i < w->end; ++i)
            w->prices[i] = bso_price_ref(w->s[i], w->k[i], w->r[i], w->v[i],
                                         w->t[i], w->otype[i]);
        pthread_mutex_lock(&g->mu);
        ++g->ndone;
        pthread_cond_signal(&g->fin);
        pthread_mutex_unlock(&g->mu);
    }
}

static double bso_now(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

double bso_bs_map(int nthreads, int num_runs, size_t n, const float* s,
                  const float* k, const float* r, const float* v,
                  const float* t, const int32_t* otype, float* prices)
{
    if (nthreads < 1 || num_runs < 0) return -1.0;
    if (n == 0) return 0.0;
    /* blackscholes.c:706-709: never more workers than options */
    if ((size_t)nthreads > n) nthreads = (int)n;

    int64_t* b = (int64_t*)malloc(sizeof(int64_t) * (size_t)nthreads);
    int64_t* e = (int64_t*)malloc(sizeof(int64_t) * (size_t)nthreads);
    bso_worker* ws = (bso_worker*)calloc((size_t)nthreads, sizeof(bso_worker));
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    if (!b || !e || !ws || !th) {
        free(b); free(e); free(ws); free(th);
        return -1.0;
    }
    bso_static_partition((int64_t)n, nthreads, b, e);

    bso_gate g;
    pthread_mutex_init(&g.mu, NULL);
    pthread_cond_init(&g.go, NULL);
    pthread_cond_init(&g.fin, NULL);
    g.gen = 0;
    g.ndone = 0;
    g.quit = 0;

    int spawned = 0;
    for (int w = 0; w < nthreads; ++w) {
        ws[w] = (bso_worker){&g, b[w], e[w], s, k, r, v, t, otype, prices};
        if (pthread_create(&th[w], NULL, bso_worker_main, &ws[w]) != 0) break;
        ++spawned;
    }
    double secs = -1.0;
    if (spawned == nthreads) {
        const double t0 = bso_now();
        for (int j = 0; j < num_runs; ++j) {
            pthread_mutex_lock(&g.mu);
            g.ndone = 0;
            g.gen++;
            pthread_cond_broadcast(&g.go);
            while (g.ndone < nthreads) pthread_cond_wait(&g.fin, &g.mu);
            pthread_mutex_unlock(&g.mu);
        }
        secs = bso_now() - t0;
    }
    pthread_mutex_lock(&g.mu);
    g.quit = 1;
    pthread_cond_broadcast(&g.go);
    pthread_mutex_unlock(&g.mu);
    for (int w = 0; w < spawned; ++w) pthread_join(th[w], NULL);

    pthread_cond_destroy(&g.go);
    pthread_cond_destroy(&g.fin);
    pthread_mutex_destroy(&g.mu);
    free(b); free(e); free(ws); free(th);
    return secs;
}

/* ---- the reference's file I/O, sequential (the I/O baseline) ------------- */

/* blackscholes.c:695-767: fscanf the count and 9 fields per option, then the
 * SoA build.  Arrays must hold n entries; returns n, or -1 on a read error. */
long bso_read_parsec_fscanf(const char* path, size_t cap, float* s, float* k,
                            float* r, float* v, float* t, int32_t* otype,
                            float* dgrefval)
{
    FILE* f = fopen(path, "r");
    if (!f) return -1;
    int n = 0;
    if (fscanf(f, "%i", &n) != 1 || n < 0 || (size_t)n > cap) {
        fclose(f);
        return -1;
    }
    for (int i = 0; i < n; ++i) {
        float divq, divs;
        char type;
        if (fscanf(f, "%f %f %f %f %f %f %c %f %f", &s[i], &k[i], &r[i], &divq,
                   &v[i], &t[i], &type, &divs, &dgrefval[i]) != 9) {
            fclose(f);
            return -1;
        }
        otype[i] = (type == 'P') ? 1 : 0;
    }
    fclose(f);
    return n;
}

/* blackscholes.c:923-947 */
int bso_write_prices_fprintf(const char* path, const float* prices, size_t n)
{
    FILE* f = fopen(path, "w");
    if (!f) return -1;
    if (fprintf(f, "%i\n", (int)n) < 0) {
        fclose(f);
        return -1;
    }
    for (size_t i = 0; i < n; ++i)
        if (fprintf(f, "%.18f\n", prices[i]) < 0) {
            fclose(f);
            return -1;
        }
    return fclose(f) == 0 ? 0 : -1;
}

/* FP64 over double inputs: the storage of the SIMD variant's NCO = 2 build
 * (blackscholes.simd.c:68-81) */
void bso_price_fp64_soa_d(size_t n, const double* s, const double* k, const double* r,
                          const double* v, const double* t, const int32_t* otype,
                          double* prices)
{
    for (size_t i = 0; i < n; ++i)
        prices[i] = bso_price_fp64(s[i], k[i], r[i], v[i], t[i], otype[i]);
}
