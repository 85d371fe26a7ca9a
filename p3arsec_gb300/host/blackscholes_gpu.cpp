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

// OptionData (blackscholes.c:89-100) is the parsed bsg_book: the five SoA
// arrays, otype and the DGrefval column (divq and divs are unused).
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

    // Parse in parallel with the reference's field conversions
    // (blackscholes.c:695-739); bsg_read_parsec fails where fscanf would.
    bsg_book book;
    {
        FILE* probe = fopen(inputFile, "r");
        if (probe == NULL) {
            printf("ERROR: Unable to open file `%s'.\n", inputFile);
            exit(1);
        }
        fclose(probe);
    }
    if (bsg_read_parsec(inputFile, 0, &book) != BSG_OK) {
        printf("ERROR: Unable to read from file `%s'.\n", inputFile);
        exit(1);
    }
    numOptions = (int)book.n;
    if (nThreads > numOptions) {
        printf("WARNING: Not enough work, reducing number of threads to match number of options.\n");
        nThreads = numOptions;
    }
    printf("Num of Options: %d\n", numOptions);
    printf("Num of Runs: %d\n", numRuns);

    // SoA in pinned memory (blackscholes.c:747-767 layout: one buffer of 5N
    // floats, otype separate)
    const size_t n = (size_t)numOptions;
    prices = (fptype*)bsg_host_alloc(sizeof(fptype) * (n ? n : 1));
    fptype* buffer = (fptype*)bsg_host_alloc(5 * sizeof(fptype) * (n ? n : 1));
    otype = (int*)bsg_host_alloc(sizeof(int) * (n ? n : 1));
    if (!buffer || !otype || !prices) {
        printf("ERROR: out of pinned memory\n");
        exit(1);
    }
    sptprice = buffer;
    strike = sptprice + n;
    rate = strike + n;
    volatility = rate + n;
    otime = volatility + n;
    if (n) {
        memcpy(sptprice, book.sptprice, n * sizeof(fptype));
        memcpy(strike, book.strike, n * sizeof(fptype));
        memcpy(rate, book.rate, n * sizeof(fptype));
        memcpy(volatility, book.volatility, n * sizeof(fptype));
        memcpy(otime, book.otime, n * sizeof(fptype));
        memcpy(otype, book.otype, n * sizeof(int));
    }
    // the reference prints numOptions * (sizeof(OptionData) + sizeof(int)),
    // with sizeof(OptionData) = 36 (8 floats and a padded char)
    printf("Size of data: %zu\n", n * (36 + sizeof(int)));

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
            const fptype priceDelta = book.dgrefval[i] - prices[i];
            if (fabs(priceDelta) >= 1e-4) {
                printf("Error on %zu. Computed=%.5f, Ref=%.5f, Delta=%.5f\n", i, prices[i],
                       book.dgrefval[i], priceDelta);
                numError++;
            }
        }
    }

    // "%i\n" then "%.18f\n" per price, formatted in parallel, byte-identical
    // to the reference's fprintf (blackscholes.c:923-947)
    if (bsg_write_parsec_prices(outputFile, prices, n, 0) != BSG_OK) {
        printf("ERROR: Unable to write to file `%s'.\n", outputFile);
        exit(1);
    }
    if (errChk) printf("Num Errors: %d\n", numError);
    bsg_destroy(ctx);
    bsg_host_free(buffer);
    bsg_host_free(otype);
    bsg_host_free(prices);
    bsg_book_free(&book);
    return 0;
}
