// swaptions_gpu.cpp -- drop-in replacement of the reference's swaptions
// driver (parsec-ff/pkgs/apps/swaptions/src/HJM_Securities.cpp:153-378)
// whose pricing runs on the GPU through libbsgpu.so.
//
//   swaptions_gpu -ns <swaptions> -sm <simulations> [-nt <threads>] [-sd <seed>]
//
// Same options, same stdout lines ("PARSEC Benchmark Suite", "Number of
// Simulations: ...") and the same per-swaption stderr line
// ("Swaption %d: [SwaptionPrice: %.10lf StdError: %.10lf]",
// HJM_Securities.cpp:353-356), plus the ROI's "roi.time|<s>" line.  The
// swaption set is the reference's (HJM_Securities.cpp:231-296): an 11-point
// grid, the three factors' vol table, the yield curve 0.1 + 0.005 j,
// maturity 1, tenor 2, annual payments, continuously compounded strikes,
// a horizon of 5 + 0.25 int(60 u) years and a strike of 0.1 + 0.1 int(49 u).
// The reference draws u with its RanUnif, which is not in its tree; here u
// comes from a splitmix64 stream seeded with -sd (u = top 53 bits / 2^53),
// drawn in the reference's order: first the base of the swaptions' seeds,
// 2147483647 u (HJM_Securities.cpp:198), then per swaption the horizon and
// the strike.  Swaption i's paths use seed base + i.  -nt is accepted for
// command-line compatibility; every swaption is priced in one GPU call.
// Errors print a message and exit(1), as the reference does.
#include "bsg.h"

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace {

struct SplitMix64 {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double unit() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

void usage(const char* name) {
    fprintf(stderr, "Usage: %s OPTION [OPTIONS]...\n", name);
    fprintf(stderr, "Options:\n");
    fprintf(stderr, "\t-ns [number of swaptions (should be > number of threads]\n");
    fprintf(stderr, "\t-sm [number of simulations]\n");
    fprintf(stderr, "\t-nt [number of threads]\n");
    fprintf(stderr, "\t-sd [random number seed]\n");
}

}  // namespace

int main(int argc, char** argv) {
    printf("PARSEC Benchmark Suite\n");
    fflush(nullptr);
    if (argc == 1) {
        usage(argv[0]);
        exit(1);
    }
    long trials = 10000, seed = 1979;
    int nthreads = 1, nsw = 1;
    for (int j = 1; j < argc; j++) {
        if (!strcmp("-sm", argv[j]) && j + 1 < argc) trials = atol(argv[++j]);
        else if (!strcmp("-nt", argv[j]) && j + 1 < argc) nthreads = atoi(argv[++j]);
        else if (!strcmp("-ns", argv[j]) && j + 1 < argc) nsw = atoi(argv[++j]);
        else if (!strcmp("-sd", argv[j]) && j + 1 < argc) seed = atol(argv[++j]);
        else {
            fprintf(stderr, "Error: Unknown option: %s\n", argv[j]);
            usage(argv[0]);
            exit(1);
        }
    }
    if (nsw < nthreads) {
        fprintf(stderr, "Error: Fewer swaptions than threads.\n");
        usage(argv[0]);
        exit(1);
    }
    if (nsw < 1 || trials < 2) {
        fprintf(stderr, "Error: need at least one swaption and two simulations.\n");
        exit(1);
    }
    printf("Number of Simulations: %ld,  Number of threads: %d Number of swaptions: %d\n", trials,
           nthreads, nsw);

    // the reference's swaption set (HJM_Securities.cpp:231-296)
    const int iN = 11, iFactors = 3;
    static const double factors[3][10] = {
        {.01, .01, .01, .01, .01, .01, .01, .01, .01, .01},
        {.009048, .008187, .007408, .006703, .006065, .005488, .004966, .004493, .004066, .003679},
        {.001000, .000750, .000500, .000250, .000000, -.000250, -.000500, -.000750, -.001000,
         -.001250}};
    std::vector<double> yield(iN);
    yield[0] = .1;
    for (int j = 1; j < iN; ++j) yield[j] = yield[j - 1] + .005;  // :288-290
    SplitMix64 rng{(uint64_t)seed};
    const uint64_t base = (uint64_t)(2147483647L * rng.unit());
    std::vector<bsg_swaption> sw(nsw);
    for (int i = 0; i < nsw; ++i) {
        bsg_swaption& w = sw[i];
        w.years = 5.0 + ((int)(60 * rng.unit())) * 0.25;
        w.strike = 0.1 + ((int)(49 * rng.unit())) * 0.1;
        w.compounding = 0;
        w.maturity = 1.0;
        w.tenor = 2.0;
        w.payment_interval = 1.0;
        w.n_steps = iN;
        w.n_factors = iFactors;
        w.yield = yield.data();
        w.factors = &factors[0][0];
        w.seed = base + (uint64_t)i;
    }

    bsg_ctx* ctx = nullptr;
    int st = bsg_create(&ctx, 0, 1);
    if (st != BSG_OK) {
        printf("ERROR: no usable GPU: %s\n", bsg_strerror(st));
        exit(1);
    }
    std::vector<double> price(nsw), err(nsw);
    const auto t0 = std::chrono::steady_clock::now();  // __parsec_roi_begin
    st = bsg_price_swaptions(ctx, sw.data(), (size_t)nsw, (uint64_t)trials, price.data(), err.data());
    const auto t1 = std::chrono::steady_clock::now();  // __parsec_roi_end
    if (st != BSG_OK) {
        printf("ERROR: %s\n", bsg_last_error(ctx));
        exit(1);
    }
    printf("roi.time|%.6f\n", std::chrono::duration<double>(t1 - t0).count());
    for (int i = 0; i < nsw; i++)
        fprintf(stderr, "Swaption %d: [SwaptionPrice: %.10lf StdError: %.10lf] \n", i, price[i],
                err[i]);
    bsg_destroy(ctx);
    return 0;
}
