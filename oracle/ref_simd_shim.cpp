/*
 * ref_simd_shim.cpp -- C entry points into the reference's SIMD variant
 * (TEST INFRASTRUCTURE ONLY).
 *
 * Linked with the reference's blackscholes.simd.c compiled unmodified from
 * its source tree with NCO = 4 (SSE, fptype float) or NCO = 2 (SSE2, fptype
 * double), main renamed.  Its BlkSchlsEqEuroNoDiv (blackscholes.simd.c:221)
 * prices one packet of NCO options from 16-byte aligned arrays; the wrapper
 * walks whole arrays packet by packet.
 */
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#if NCO == 4
typedef float fptype;
#define BSREF_SIMD_PRICE bsref_simd4_price
#else
typedef double fptype;
#define BSREF_SIMD_PRICE bsref_simd2_price
#endif

void BlkSchlsEqEuroNoDiv(fptype* OptionPrice, int numOptions, fptype* sptprice,
                         fptype* strike, fptype* rate, fptype* volatility,
                         fptype* time, int* otype, float timet);

extern "C" void BSREF_SIMD_PRICE(size_t n, const fptype* s, const fptype* k,
                                 const fptype* r, const fptype* v, const fptype* t,
                                 const int32_t* otype, fptype* prices)
{
    alignas(16) fptype bs[NCO], bk[NCO], br[NCO], bv[NCO], bt[NCO], out[NCO];
    alignas(16) int bo[NCO];
    for (size_t i = 0; i < n; i += NCO) {
        const size_t m = (n - i < NCO) ? n - i : NCO;
        for (size_t j = 0; j < NCO; ++j) {  // pad a short last packet
            const size_t q = i + (j < m ? j : 0);
            bs[j] = s[q]; bk[j] = k[q]; br[j] = r[q]; bv[j] = v[q]; bt[j] = t[q];
            bo[j] = otype[q];
        }
        BlkSchlsEqEuroNoDiv(out, NCO, bs, bk, br, bv, bt, bo, 0);
        for (size_t j = 0; j < m; ++j) prices[i + j] = out[j];
    }
}
