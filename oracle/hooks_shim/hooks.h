/*
 * hooks.h -- stand-in for PARSEC's hooks header (TEST INFRASTRUCTURE ONLY).
 *
 * PARSEC's own hooks library (parsec-hooks/pkgs/libs/hooks/src/hooks.c) comes
 * with the PARSEC download and Mammut, neither of which is available.  This
 * header gives the reference's blackscholes.c the four hook calls it makes
 * (blackscholes.c:682-684, 781-783, 912-914, 955-957) with the ROI timing
 * semantics of hooks.c:185-262: wall time between roi_begin and roi_end,
 * printed as "roi.time|<seconds>" (hooks.c:243).  No energy counters.
 */
#ifndef BSO_HOOKS_SHIM_H
#define BSO_HOOKS_SHIM_H

#include <stdio.h>
#include <time.h>

enum __parsec_benchmark { __parsec_blackscholes = 0 };

static double __bso_roi_t0;

static inline double __bso_hooks_now(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static inline void __parsec_bench_begin(enum __parsec_benchmark b)
{
    (void)b;
    printf("[HOOKS] PARSEC Hooks shim\n");
    fflush(NULL);
}

static inline void __parsec_roi_begin(void)
{
    printf("[HOOKS] Entering ROI\n");
    fflush(NULL);
    __bso_roi_t0 = __bso_hooks_now();
}

static inline void __parsec_roi_end(void)
{
    const double d = __bso_hooks_now() - __bso_roi_t0;
    printf("roi.time|%.9f\n", d);
    fflush(NULL);
}

static inline void __parsec_bench_end(void)
{
    printf("[HOOKS] Leaving ROI\n");
    fflush(NULL);
}

#endif
