/* A caller written against the reference's batch signature
 * (blackscholes.simd.c:221-223), built against include/bsg_compat.h and
 * linked with libbsgpu.so.  It prices n options twice: in one call, and in
 * packets of NCO = 4 as the reference's bs_thread does (blackscholes.simd.c:
 * 376-383), then prints every price of both runs as its float bit pattern.
 *
 * Usage: compat_caller <input.bin>  where the file holds n (int32) then the
 * five float arrays and the int32 otype array of n options each. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "bsg_compat.h"

#define NCO 4

static void* read_array(FILE* f, size_t bytes) {
    void* p = malloc(bytes ? bytes : 1);
    if (!p || fread(p, 1, bytes, f) != bytes) {
        fprintf(stderr, "short input\n");
        exit(2);
    }
    return p;
}

int main(int argc, char** argv) {
    if (argc != 2) return 2;
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 2;
    int32_t n = 0;
    if (fread(&n, 4, 1, f) != 1 || n < 0 || n % NCO) return 2;
    const size_t b = (size_t)n * 4;
    float* sptprice = (float*)read_array(f, b);
    float* strike = (float*)read_array(f, b);
    float* rate = (float*)read_array(f, b);
    float* volatility = (float*)read_array(f, b);
    float* otime = (float*)read_array(f, b);
    int* otype = (int*)read_array(f, b);
    fclose(f);
    float* whole = (float*)malloc(b ? b : 1);
    float* packets = (float*)malloc(b ? b : 1);
    float price[NCO];

    BlkSchlsEqEuroNoDiv(whole, n, sptprice, strike, rate, volatility, otime, otype, 0);
    for (int i = 0; i < n; i += NCO) {
        BlkSchlsEqEuroNoDiv(price, NCO, &sptprice[i], &strike[i], &rate[i], &volatility[i],
                            &otime[i], &otype[i], 0);
        for (int k = 0; k < NCO; k++) packets[i + k] = price[k];
    }
    for (int i = 0; i < n; i++) {
        uint32_t u, v;
        memcpy(&u, &whole[i], 4);
        memcpy(&v, &packets[i], 4);
        printf("%08x %08x\n", u, v);
    }
    return 0;
}
