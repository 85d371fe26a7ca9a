/*
 * bsg_compat.h -- the reference's batch signature, for a source-level drop-in.
 *
 * The SIMD variant of P3ARSEC's blackscholes prices options through
 *
 *     void BlkSchlsEqEuroNoDiv(fptype* OptionPrice, int numOptions,
 *                              fptype* sptprice, fptype* strike, fptype* rate,
 *                              fptype* volatility, fptype* time, int* otype,
 *                              float timet);
 *
 * (parsec-ff/pkgs/apps/blackscholes/src/blackscholes.simd.c:221-223, called
 * from bs_thread at :379-380 once per NCO options).  A caller that includes
 * this header in place of its own definition of that function keeps every
 * call site unchanged and prices on the GPU through libbsgpu.so
 * (bsg_BlkSchlsEqEuroNoDiv: one pass, host pointers, the default context of
 * device 0).  fptype must be float (the NCO = 4 build), as in bsg.h.
 *
 * The reference's function returns nothing and its program exits on fatal
 * errors (blackscholes.c:697-739); this wrapper does the same: on a failed
 * call it prints the library's status to stderr and calls exit(1).  Callers
 * that want the status use bsg_BlkSchlsEqEuroNoDiv directly.
 *
 * Link with -lbsgpu.
 */
#ifndef BSG_COMPAT_H
#define BSG_COMPAT_H

#include <stdio.h>
#include <stdlib.h>

#include "bsg.h"

#ifdef __cplusplus
extern "C" {
#endif

static inline void BlkSchlsEqEuroNoDiv(float* OptionPrice, int numOptions, float* sptprice,
                                       float* strike, float* rate, float* volatility,
                                       float* time, int* otype, float timet) {
    const int st = bsg_BlkSchlsEqEuroNoDiv(OptionPrice, numOptions, sptprice, strike, rate,
                                           volatility, time, otype, timet);
    if (st != BSG_OK) {
        fprintf(stderr, "BlkSchlsEqEuroNoDiv: %s\n", bsg_strerror(st));
        exit(1);
    }
}

#ifdef __cplusplus
}
#endif
#endif /* BSG_COMPAT_H */
