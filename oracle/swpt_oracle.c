/*
 * swpt_oracle.c -- CPU oracle for the swaption Monte Carlo (TEST
 * INFRASTRUCTURE ONLY; see swpt_oracle.h for what is restated from where).
 * Parity with the reference is unpinned: its model core is not in the
 * reference tree.
 */
#include "swpt_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define SWO_MAX_STEPS 32
#define SWO_MAX_FACTORS 8

/* ---- Philox4x32-10 (Salmon et al., SC'11) -------------------------------- */
static void mulhilo32(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo) {
    const uint64_t p = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(p >> 32);
    *lo = (uint32_t)p;
}

void swo_philox4x32_10(const uint32_t c[4], const uint32_t k[2], uint32_t out[4]) {
    uint32_t x0 = c[0], x1 = c[1], x2 = c[2], x3 = c[3];
    uint32_t k0 = k[0], k1 = k[1];
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        mulhilo32(0xD2511F53u, x0, &hi0, &lo0);
        mulhilo32(0xCD9E8D57u, x2, &hi1, &lo1);
        const uint32_t y0 = hi1 ^ x1 ^ k0, y1 = lo1, y2 = hi0 ^ x3 ^ k1, y3 = lo0;
        x0 = y0;
        x1 = y1;
        x2 = y2;
        x3 = y3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = x0;
    out[1] = x1;
    out[2] = x2;
    out[3] = x3;
}

/* (0, 1) from 52 random bits k (the top 20 bits of a, all of b): the double
 * 1 + k 2^-52 built from its bits, minus 1 (exact), plus 2^-53 (exact):
 * (2k + 1) 2^-53. */
static double unit52(uint32_t a, uint32_t b) {
    const uint64_t bits = 0x3FF0000000000000ull | ((uint64_t)(a >> 12) << 32) | b;
    double d;
    memcpy(&d, &bits, sizeof d);
    return (d - 1.0) + 1.1102230246251565e-16;
}

void swo_normal_pair(uint64_t seed, uint64_t trial, uint32_t j, double z[2]) {
    const uint32_t c[4] = {(uint32_t)trial, (uint32_t)(trial >> 32), j, 0u};
    const uint32_t k[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t x[4];
    swo_philox4x32_10(c, k, x);
    const double u1 = unit52(x[0], x[1]), u2 = unit52(x[2], x[3]);
    const double r = sqrt(-2.0 * log(u1));
    const double th = 6.283185307179586 * u2;
    z[0] = r * cos(th);
    z[1] = r * sin(th);
}

/* ---- model core ---------------------------------------------------------- */
void swo_yield_to_forward(int n, const double* y, double* f) {
    f[0] = y[0];
    for (int i = 1; i < n; ++i) f[i] = (double)(i + 1) * y[i] - (double)i * y[i - 1];
}

void swo_drift(int n, int nf, const double* v, double h, double* mu) {
    for (int m = 0; m < n - 1; ++m) mu[m] = 0.0;
    for (int k = 0; k < nf; ++k) {
        double s_prev = 0.0;  /* S_k(m - 1) */
        for (int m = 0; m < n - 1; ++m) {
            const double vk = v[k * (n - 1) + m];
            /* (S(m)^2 - S(m-1)^2) / 2 = vk (S(m-1) + vk / 2) */
            mu[m] += h * vk * (s_prev + 0.5 * vk);
            s_prev += vk;
        }
    }
}

/* The driver's per-swaption constants (HJM_Swaption_Blocking.cpp:48-62,
 * 116-140): step, strike in continuous compounding, indices, swap payments. */
typedef struct swo_setup {
    double h, strike_cont;
    int freq, swap_len, start, swap_points;
    double payoffs[SWO_MAX_STEPS];
} swo_setup;

static int setup(const swo_swaption* sw, swo_setup* st) {
    const int n = sw->n_steps;
    if (n < 2 || n > SWO_MAX_STEPS || sw->n_factors < 1 || sw->n_factors > SWO_MAX_FACTORS)
        return 0;
    st->h = sw->years / n;                                                  /* :48 */
    st->freq = (int)(sw->payment_interval / st->h + 0.5);                   /* :50 */
    st->strike_cont = sw->compounding == 0
                          ? sw->strike                                       /* :56-62 */
                          : (1 / sw->compounding) * log(1 + sw->strike * sw->compounding);
    st->swap_len = (int)(n - sw->maturity / st->h + 0.5);                   /* :116 */
    st->start = (int)(sw->maturity / st->h + 0.5);                          /* :125 */
    st->swap_points = (int)(sw->tenor / st->h + 0.5);                       /* :126 */
    /* the reference writes payoffs[i] for i up to swap_points and reads the
     * path's row `start`: both must stay inside the arrays it allocates */
    if (st->freq < 1 || st->start < 1 || st->start > n - 1 || st->swap_len < 1 ||
        st->swap_len > n - st->start || st->swap_points >= st->swap_len)
        return 0;
    for (int i = 0; i < st->swap_len; ++i) st->payoffs[i] = 0.0;            /* :132-133 */
    for (int i = st->freq; i <= st->swap_points; i += st->freq) {           /* :134-140 */
        if (i != st->swap_points) st->payoffs[i] = exp(st->strike_cont * sw->payment_interval) - 1;
        if (i == st->swap_points) st->payoffs[i] = exp(st->strike_cont * sw->payment_interval);
    }
    return 1;
}

int swo_price(const swo_swaption* sw, uint64_t trials, unsigned flags, double out[2]) {
    swo_setup st;
    if (!setup(sw, &st) || trials < 2) return 0;
    const int n = sw->n_steps, nf = sw->n_factors;
    const double h = st.h, sqh = sqrt(h);
    double fwd[SWO_MAX_STEPS], mu[SWO_MAX_STEPS];
    swo_yield_to_forward(n, sw->yield, fwd);
    swo_drift(n, nf, sw->factors, h, mu);
    /* path[i][m] = f(t_i, t_{i+m}), m < n - i */
    double path[SWO_MAX_STEPS][SWO_MAX_STEPS];
    double z[SWO_MAX_STEPS * SWO_MAX_FACTORS + 2];
    const int nz = (n - 1) * nf;
    double sum = 0.0, sum_sq = 0.0;
    for (uint64_t t = 0; t < trials; ++t) {
        for (int q = 0; q < nz; q += 2) swo_normal_pair(sw->seed, t, (uint32_t)(q / 2), z + q);
        for (int m = 0; m < n; ++m) path[0][m] = fwd[m];
        /* the whole path matrix, every step (the reference simulates all of it) */
        for (int i = 0; i < n - 1; ++i)
            for (int m = 0; m < n - 1 - i; ++m) {
                double shock = 0.0;
                for (int k = 0; k < nf; ++k) shock += sw->factors[k * (n - 1) + m] * z[i * nf + k];
                path[i + 1][m] = path[i][m + 1] + mu[m] * h + sqh * shock;
            }
        /* discount to the swaption's maturity along the short rates, and the
         * swap's discount factors along the forward curve at maturity
         * (HJM_Swaption_Blocking.cpp:165-184) */
        double acc = 0.0;
        for (int i = 0; i < st.start; ++i) acc += path[i][0];
        const double disc = exp(-acc * h);
        double fixed = 0.0, accs = 0.0;                                     /* :191-195 */
        for (int l = 0; l < st.swap_len; ++l) {
            fixed += st.payoffs[l] * exp(-accs * h);
            accs += path[st.start][l];
        }
        const double payoff = (flags & 1u) ? fixed - 1.0 : (fixed - 1.0 > 0 ? fixed - 1.0 : 0.0);
        const double dp = payoff * disc;                                     /* :196-198 */
        sum += dp;                                                           /* :203-204 */
        sum_sq += dp * dp;
    }
    out[0] = sum / (double)trials;                                           /* :212-214 */
    out[1] = sqrt((sum_sq - sum * sum / (double)trials) / ((double)trials - 1.0)) /
             sqrt((double)trials);
    return 1;
}

/* ---- the ParallelFor over swaptions -------------------------------------- */
typedef struct swo_job {
    const swo_swaption* sw;
    int begin, end;
    uint64_t trials;
    double *price, *err;
    int ok;
} swo_job;

static void* swo_worker(void* arg) {
    swo_job* j = (swo_job*)arg;
    j->ok = 1;
    for (int i = j->begin; i < j->end; ++i) {
        double o[2] = {NAN, NAN};
        if (!swo_price(&j->sw[i], j->trials, 0, o)) j->ok = 0;
        j->price[i] = o[0];
        j->err[i] = o[1];
    }
    return NULL;
}

double swo_price_all(const swo_swaption* sw, int n, uint64_t trials, int nthreads,
                     double* price, double* err) {
    if (n < 0 || nthreads < 1) return -1.0;
    if (nthreads > n) nthreads = n > 0 ? n : 1;
    swo_job* jobs = (swo_job*)calloc((size_t)nthreads, sizeof(swo_job));
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    if (!jobs || !th) {
        free(jobs);
        free(th);
        return -1.0;
    }
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    /* FastFlow's default static partition: blocks of n / nw, the first
     * n % nw one larger */
    const int q = n / nthreads, r = n % nthreads;
    int b = 0, failed = 0;
    for (int w = 0; w < nthreads; ++w) {
        const int len = q + (w < r ? 1 : 0);
        jobs[w] = (swo_job){sw, b, b + len, trials, price, err, 0};
        b += len;
        if (pthread_create(&th[w], NULL, swo_worker, &jobs[w]) != 0) {
            th[w] = 0;
            swo_worker(&jobs[w]);  /* no thread: price this block here */
        }
    }
    for (int w = 0; w < nthreads; ++w)
        if (th[w]) pthread_join(th[w], NULL);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    for (int w = 0; w < nthreads; ++w)
        if (!jobs[w].ok) failed = 1;
    free(jobs);
    free(th);
    if (failed) return -1.0;
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}
