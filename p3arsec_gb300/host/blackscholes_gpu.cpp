// blackscholes_gpu.cpp -- drop-in replacement of the reference's blackscholes
// driver (parsec-ff/pkgs/apps/blackscholes/src/blackscholes.c:664-961) whose
// hot loop runs on the GPU through libbsgpu.so.
//
//   blackscholes_gpu <nthreads> <inputFile> <outputFile>
//
// Same input format (count, then "%f %f %f %f %f %f %c %f %f" per option),
// same output format ("%i\n" then "%.18f\n" per price), same stdout lines
// (Num of Options, Num of Runs, Size of data, roi.time|<s>).  <nthreads> is
// accepted for command-line compatibility; the GPU map does not use host
// threads.  Environment: BSG_ERR_CHK=1 compares every price with the
// DGrefval column at the reference's 1e-4 threshold and prints Num Errors
// (blackscholes.c:333-339, 949-951); BSG_NUM_RUNS overrides NUM_RUNS;
// BSG_MODE = fast | sfu_ref | libm_ref selects the arithmetic.
// Errors print a message and exit(1), as the reference does.
#include "bsg.h"

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#define fptype float
#define NUM_RUNS BSG_NUM_RUNS

typedef struct OptionData_ {  // blackscholes.c:89-100
    fptype s, strike, r, divq, v, t;
    char OptionType;
    fptype divs, DGrefval;
} OptionData;

static OptionData* data;
static fptype* prices;
static int numOptions;
static int* otype;
static fptype *sptprice, *strike, *rate, *volatility, *otime;
static int numError = 0;
static int nThreads;
static int numRuns = NUM_RUNS;
static unsigned modeFlag = BSG_MODE_FAST;
static bsg_ctx* ctx;

// blackscholes.simd.c:221-223 batch signature, priced once on the GPU.
void BlkSchlsEqEuroNoDiv(fptype* OptionPrice, int numOptions, fptype* sptprice,
                         fptype* strike, fptype* rate, fptype* volatility,
                         fptype* time, int* otype, float timet) {
    int st = bsg_BlkSchlsEqEuroNoDiv(OptionPrice, numOptions, sptprice, strike, rate,
                                     volatility, time, otype, timet);
    if (st != BSG_OK) {
        printf("ERROR: GPU pricing failed: %s\n", bsg_strerror(st));
        exit(1);
    }
}

// blackscholes.c:607-658: NUM_RUNS passes over all options.  One call covers
// every option (the GPU grid replaces the per-thread ranges).
int bs_thread(void* tid_ptr) {
    (void)tid_ptr;
    int st = bsg_price_soa(ctx, sptprice, strike, rate, volatility, otime,
                           (const int32_t*)otype, prices, (size_t)numOptions, numRuns,
                           BSG_HOST_PTRS | modeFlag);
    if (st != BSG_OK) {
        printf("ERROR: GPU pricing failed: %s (%s)\n", bsg_strerror(st), bsg_last_error(ctx));
        exit(1);
    }
    return 0;
}

int main(int argc, char** argv) {
    printf("PARSEC Benchmark Suite\n");
    fflush(NULL);
    if (argc != 4) {
        printf("Usage:\n\t%s <nthreads> <inputFile> <outputFile>\n", argv[0]);
        exit(1);
    }
    nThreads = atoi(argv[1]);
    const char* inputFile = argv[2];
    const char* outputFile = argv[3];
    if (const char* e = getenv("BSG_NUM_RUNS")) numRuns = atoi(e);
    if (const char* e = getenv("BSG_MODE")) {
        if (!strcmp(e, "sfu_ref")) modeFlag = BSG_MODE_SFU_REF;
        else if (!strcmp(e, "libm_ref")) modeFlag = BSG_MODE_LIBM_REF;
    }
    const bool errChk = getenv("BSG_ERR_CHK") && atoi(getenv("BSG_ERR_CHK")) != 0;

    FILE* file = fopen(inputFile, "r");
    if (file == NULL) {
        printf("ERROR: Unable to open file `%s'.\n", inputFile);
        exit(1);
    }
    if (fscanf(file, "%i", &numOptions) != 1 || numOptions < 0) {
        printf("ERROR: Unable to read from file `%s'.\n", inputFile);
        fclose(file);
        exit(1);
    }
    if (nThreads > numOptions) {
        printf("WARNING: Not enough work, reducing number of threads to match number of options.\n");
        nThreads = numOptions;
    }
    data = (OptionData*)malloc(sizeof(OptionData) * (size_t)(numOptions ? numOptions : 1));
    prices = (fptype*)bsg_host_alloc(sizeof(fptype) * (size_t)(numOptions ? numOptions : 1));
    if (!data || !prices) {
        printf("ERROR: out of memory\n");
        exit(1);
    }
    for (int i = 0; i < numOptions; ++i) {
        int rv = fscanf(file, "%f %f %f %f %f %f %c %f %f", &data[i].s, &data[i].strike,
                        &data[i].r, &data[i].divq, &data[i].v, &data[i].t,
                        &data[i].OptionType, &data[i].divs, &data[i].DGrefval);
        if (rv != 9) {
            printf("ERROR: Unable to read from file `%s'.\n", inputFile);
            fclose(file);
            exit(1);
        }
    }
    if (fclose(file) != 0) {
        printf("ERROR: Unable to close file `%s'.\n", inputFile);
        exit(1);
    }
    printf("Num of Options: %d\n", numOptions);
    printf("Num of Runs: %d\n", numRuns);

    // SoA in pinned memory (blackscholes.c:747-767 layout: one buffer of 5N
    // floats, otype separate)
    const size_t n = (size_t)numOptions;
    fptype* buffer = (fptype*)bsg_host_alloc(5 * sizeof(fptype) * (n ? n : 1));
    otype = (int*)bsg_host_alloc(sizeof(int) * (n ? n : 1));
    if (!buffer || !otype) {
        printf("ERROR: out of pinned memory\n");
        exit(1);
    }
    sptprice = buffer;
    strike = sptprice + n;
    rate = strike + n;
    volatility = rate + n;
    otime = volatility + n;
    for (size_t i = 0; i < n; ++i) {
        otype[i] = (data[i].OptionType == 'P') ? 1 : 0;
        sptprice[i] = data[i].s;
        strike[i] = data[i].strike;
        rate[i] = data[i].r;
        volatility[i] = data[i].v;
        otime[i] = data[i].t;
    }
    printf("Size of data: %zu\n", n * (sizeof(OptionData) + sizeof(int)));

    int st = bsg_create(&ctx, 0, n ? n : 1);
    if (st != BSG_OK) {
        printf("ERROR: no usable GPU: %s\n", bsg_strerror(st));
        exit(1);
    }

    printf("[HOOKS] Entering ROI\n");
    fflush(NULL);
    const auto t0 = std::chrono::steady_clock::now();
    int tid = 0;
    bs_thread(&tid);
    const double roi = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    printf("roi.time|%.9f\n", roi);

    if (errChk) {
        for (size_t i = 0; i < n; ++i) {
            const fptype priceDelta = data[i].DGrefval - prices[i];
            if (fabs(priceDelta) >= 1e-4) {
                printf("Error on %zu. Computed=%.5f, Ref=%.5f, Delta=%.5f\n", i, prices[i],
                       data[i].DGrefval, priceDelta);
                numError++;
            }
        }
    }

    file = fopen(outputFile, "w");
    if (file == NULL) {
        printf("ERROR: Unable to open file `%s'.\n", outputFile);
        exit(1);
    }
    if (fprintf(file, "%i\n", numOptions) < 0) {
        printf("ERROR: Unable to write to file `%s'.\n", outputFile);
        fclose(file);
        exit(1);
    }
    for (size_t i = 0; i < n; ++i) {
        if (fprintf(file, "%.18f\n", prices[i]) < 0) {
            printf("ERROR: Unable to write to file `%s'.\n", outputFile);
            fclose(file);
            exit(1);
        }
    }
    if (fclose(file) != 0) {
        printf("ERROR: Unable to close file `%s'.\n", outputFile);
        exit(1);
    }
    if (errChk) printf("Num Errors: %d\n", numError);
    bsg_destroy(ctx);
    bsg_host_free(buffer);
    bsg_host_free(otype);
    bsg_host_free(prices);
    free(data);
    return 0;
}
