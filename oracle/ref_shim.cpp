/*
 * ref_shim.cpp -- C entry points into the reference's own pricing function
 * (TEST INFRASTRUCTURE ONLY).
 *
 * Linked with the reference's blackscholes.c, compiled unmodified from its
 * source tree (its main() renamed by -Dmain=parsec_blackscholes_main), into
 * oracle/_ref/libbsref.so.  The reference is a C++ translation unit, so its
 * functions carry C++ linkage; this file declares them and exposes unmangled
 * batch wrappers that tests call through ctypes.
 */
#include <stddef.h>
#include <stdint.h>

/* blackscholes.c:126 and :190 (fptype = float, :85) */
float CNDF(float InputX);
float BlkSchlsEqEuroNoDiv(float sptprice, float strike, float rate,
                          float volatility, float time, int otype, float timet);

extern "C" {

void bsref_price_soa(size_t n, const float* s, const float* k, const float* r,
                     const float* v, const float* t, const int32_t* otype,
                     float* prices)
{
    for (size_t i = 0; i < n; ++i)
        prices[i] = BlkSchlsEqEuroNoDiv(s[i], k[i], r[i], v[i], t[i], otype[i], 0);
}

void bsref_cndf(size_t n, const float* x, float* out)
{
    for (size_t i = 0; i < n; ++i) out[i] = CNDF(x[i]);
}

}
