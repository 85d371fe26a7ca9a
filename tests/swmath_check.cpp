// CPU check of the swaption Monte Carlo's elementary functions (the
// table-driven Box-Muller transform and exp of
// p3arsec_gb300/csrc/bsg_swmath.h, the same code the GPU runs) against
// long-double logl/sinl/cosl/expl.
//
//   swmath_check walk <n> <seed>
//       n pseudo-random 52-bit integers (splitmix64) plus the edge cases
//       (u next to 0 and 1, every table boundary of both functions and
//       its neighbours); prints one line
//       "checked <n> log_ulp <a> trig_abs <b> z_rel <c> exp_ulp <d>"
//       log_ulp: max |W - (-2 ln u)| / ulp(-2 ln u); trig_abs: max absolute
//       error of sin and cos; z_rel: max |z - exact| / max(1, |exact|);
//       exp_ulp: max |exp_(x) - e^x| / ulp(e^x) over n arguments in
//       [-40, 40], n/4 in (-700, 700) and the points k ln2/64 and their
//       neighbours.
//   swmath_check pairs <in> <out>
//       reads 4 x uint32 words per pair from <in>, writes z0, z1 (double)
//       per pair to <out>: the host side of the GPU bit-identity test.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "bsg_swmath.h"

namespace {

const bsg_sw::Tables kT = BSG_SW_TABLES;

struct SplitMix64 {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
};

double ulp(double x) { return std::nextafter(std::fabs(x), INFINITY) - std::fabs(x); }

int walk(long n, uint64_t seed) {
    const unsigned long long kMax = (1ull << 52) - 1;
    std::vector<uint64_t> ks;
    SplitMix64 g{seed};
    for (long i = 0; i < n; ++i) ks.push_back(g.next() >> 12);
    for (uint64_t k : {0ull, 1ull, 2ull, 3ull, kMax, kMax - 1, kMax - 2, 1ull << 51, (1ull << 51) - 1,
                       1ull << 50, 3ull << 50, (3ull << 50) - 1, 12345678901ull})
        ks.push_back(k);
    for (int lz = 0; lz < 52; ++lz) ks.push_back(1ull << lz), ks.push_back((1ull << lz) - 1);
    for (long j = 0; j <= 256; ++j)
        for (long d = -3; d <= 3; ++d)
            for (long edge : {0l, 1l << 43, 1l << 44})  // the 1/256 and 1/128 grids' points and midpoints
                for (long sh : {44l, 45l}) {
                    const long long k = (j << sh) + edge + d;
                    if (k >= 0 && (uint64_t)k <= kMax) ks.push_back((uint64_t)k);
                }
    const long double pi = acosl(-1.0L);
    double log_ulp = 0, trig = 0, zrel = 0;
    for (size_t i = 0; i < ks.size(); ++i) {
        const uint64_t k = ks[i], k2 = ks[(i * 7 + 3) % ks.size()];
        const long double u = (long double)(2 * k + 1) / 9007199254740992.0L;
        const long double u2 = (long double)(2 * k2 + 1) / 9007199254740992.0L;
        const long double w_ex = -2.0L * logl(u);
        const double w = bsg_sw::neg2_ln_unit(kT, k);
        log_ulp = std::fmax(log_ulp, (double)(fabsl((long double)w - w_ex) / ulp((double)w_ex)));
        double s, c;
        bsg_sw::sincos_2pi_unit(kT, k2, &s, &c);
        const long double s_ex = sinl(2 * pi * u2), c_ex = cosl(2 * pi * u2);
        trig = std::fmax(trig, (double)std::fmax(fabsl(s - s_ex), fabsl(c - c_ex)));
        double z0, z1;
        const uint32_t w0 = (uint32_t)((k >> 32) << 12), w1 = (uint32_t)k;
        const uint32_t w2 = (uint32_t)((k2 >> 32) << 12), w3 = (uint32_t)k2;
        bsg_sw::normal_pair(kT, w0, w1, w2, w3, &z0, &z1);
        const long double r = sqrtl(w_ex);
        const long double e0 = r * c_ex, e1 = r * s_ex;
        zrel = std::fmax(zrel, (double)(fabsl(z0 - e0) / fmaxl(1.0L, fabsl(e0))));
        zrel = std::fmax(zrel, (double)(fabsl(z1 - e1) / fmaxl(1.0L, fabsl(e1))));
    }
    std::vector<double> xs;
    for (long i = 0; i < n; ++i) xs.push_back(-40.0 + 80.0 * ((g.next() >> 11) * 0x1.0p-53));
    for (long i = 0; i < n / 4; ++i) xs.push_back(-699.99 + 1399.98 * ((g.next() >> 11) * 0x1.0p-53));
    for (double x : {0.0, -0.0, 1e-300, -1e-300, 1e-17, -1e-17, 699.99, -699.99, 1.0, -1.0})
        xs.push_back(x);
    const long double l64 = logl(2.0L) / 64;
    for (long k = -4096; k <= 4096; ++k) {
        const double x = (double)(k * l64);
        xs.push_back(x);
        xs.push_back(std::nextafter(x, INFINITY));
        xs.push_back(std::nextafter(x, -INFINITY));
        xs.push_back((double)((k + 0.5L) * l64));  // the rounding boundaries of k
    }
    double exp_ulp = 0;
    for (double x : xs) {
        const long double ex = expl((long double)x);
        const double got = bsg_sw::exp_(kT, x);
        exp_ulp = std::fmax(exp_ulp, (double)(fabsl((long double)got - ex) / ulp((double)ex)));
    }
    printf("checked %zu log_ulp %.4f trig_abs %.4e z_rel %.4e exp_ulp %.4f\n", ks.size() + xs.size(),
           log_ulp, trig, zrel, exp_ulp);
    return 0;
}

int pairs(const char* in, const char* out) {
    FILE* f = fopen(in, "rb");
    if (!f) return 2;
    std::vector<uint32_t> w;
    uint32_t buf[4];
    while (fread(buf, 4, 4, f) == 4) w.insert(w.end(), buf, buf + 4);
    fclose(f);
    std::vector<double> z(w.size() / 2);
    for (size_t i = 0; i < w.size() / 4; ++i)
        bsg_sw::normal_pair(kT, w[4 * i], w[4 * i + 1], w[4 * i + 2], w[4 * i + 3], &z[2 * i],
                            &z[2 * i + 1]);
    FILE* g = fopen(out, "wb");
    if (!g) return 2;
    fwrite(z.data(), 8, z.size(), g);
    fclose(g);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc == 4 && !strcmp(argv[1], "walk")) return walk(atol(argv[2]), strtoull(argv[3], nullptr, 10));
    if (argc == 4 && !strcmp(argv[1], "pairs")) return pairs(argv[2], argv[3]);
    fprintf(stderr, "usage: swmath_check walk <n> <seed> | pairs <in> <out>\n");
    return 2;
}
