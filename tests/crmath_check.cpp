// CPU check of the float-float exp and log (p3arsec_gb300/csrc/bsg_crmath.h,
// the same code the GPU's reference-order pricing runs) against long-double
// expl/logl rounded to float.
//
//   crmath_check exp|log <stride> <threads>
//   crmath_check special
//
// Walks every <stride>-th float of the function's domain (exp: [-87, 88.5];
// log: positive normal floats) and prints one line:
//   "<fn> checked <n> misrounded <m> max_ulp <u> worst_midpoint <d>"
// misrounded = results that differ from the correctly rounded float; each
// of those must be a near-midpoint case (exact value within 2^-40 relative
// of the halfway point between two floats) and at most one ulp away.
// worst_midpoint is the largest relative distance from the midpoint among
// the misrounded (0 when none).  Exit status 1 if any result is more than
// one ulp off or misrounded far from a midpoint.
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "bsg_crmath.h"

namespace {

uint32_t bits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
float from_bits(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

// ulps between two positive finite floats
int64_t ulp_dist(float a, float b) {
    return std::llabs((int64_t)bits(a) - (int64_t)bits(b));
}

struct Result {
    uint64_t checked = 0, misrounded = 0, far = 0;
    int64_t max_ulp = 0;
    long double worst_mid = 0;
};

void check_one(float x, long double exact, float got, Result& r) {
    ++r.checked;
    const float want = (float)exact;
    if (bits(got) == bits(want)) return;
    ++r.misrounded;
    // for log, results may be negative: compare magnitudes
    const float ag = std::fabs(got), aw = std::fabs(want);
    const int64_t d = ulp_dist(ag, aw);
    if (d > r.max_ulp) r.max_ulp = d;
    const long double mid = ((long double)ag + (long double)aw) / 2;
    const long double rel = std::fabs(std::fabs(exact) - mid) / std::fabs(exact);
    if (rel > r.worst_mid) r.worst_mid = rel;
    if (d > 1 || rel > 0x1p-40L) {
        ++r.far;
        if (r.far <= 5)
            std::printf("far: x=%a got=%a want=%a rel_to_mid=%Lg\n", x, got, want, rel);
    }
}

}  // namespace

// Special and out-of-domain arguments go to the platform's expf/logf and
// must come back with their IEEE results.
int check_special() {
    const float inf = INFINITY, nan = NAN;
    int bad = 0;
    auto same = [&](const char* what, float got, float want) {
        const bool ok = (std::isnan(want) && std::isnan(got)) || bits(got) == bits(want);
        if (!ok) {
            std::printf("special %s: got %a want %a\n", what, got, want);
            ++bad;
        }
    };
    same("exp(nan)", bsg_cr::exp(nan), nan);
    same("exp(-inf)", bsg_cr::exp(-inf), 0.0f);
    same("exp(inf)", bsg_cr::exp(inf), inf);
    same("exp(0)", bsg_cr::exp(0.0f), 1.0f);
    same("exp(-0)", bsg_cr::exp(-0.0f), 1.0f);
    same("exp(-100)", bsg_cr::exp(-100.0f), expf(-100.0f));
    same("exp(-104)", bsg_cr::exp(-104.0f), expf(-104.0f));
    same("exp(89)", bsg_cr::exp(89.0f), expf(89.0f));
    same("exp(88.5)", bsg_cr::exp(88.5f), (float)expl(88.5L));
    same("exp(-87)", bsg_cr::exp(-87.0f), (float)expl(-87.0L));
    same("log(nan)", bsg_cr::log(nan), nan);
    same("log(0)", bsg_cr::log(0.0f), -inf);
    same("log(-0)", bsg_cr::log(-0.0f), -inf);
    same("log(-1)", bsg_cr::log(-1.0f), nan);
    same("log(inf)", bsg_cr::log(inf), inf);
    same("log(1)", bsg_cr::log(1.0f), 0.0f);
    same("log(denorm_min)", bsg_cr::log(from_bits(1)), logf(from_bits(1)));
    same("log(subnormal)", bsg_cr::log(from_bits(0x00400000u)), logf(from_bits(0x00400000u)));
    same("log(FLT_MIN)", bsg_cr::log(from_bits(0x00800000u)), (float)logl((long double)from_bits(0x00800000u)));
    same("log(FLT_MAX)", bsg_cr::log(from_bits(0x7F7FFFFFu)), (float)logl((long double)from_bits(0x7F7FFFFFu)));
    std::printf("special checked, %d bad\n", bad);
    return bad ? 1 : 0;
}

int main(int argc, char** argv) {
    if (argc == 2 && std::strcmp(argv[1], "special") == 0) return check_special();
    if (argc != 4) {
        std::printf("usage: crmath_check exp|log <stride> <threads>\n");
        return 2;
    }
    const bool is_exp = std::strcmp(argv[1], "exp") == 0;
    const uint32_t stride = (uint32_t)std::strtoul(argv[2], nullptr, 10);
    const int nthreads = std::atoi(argv[3]);
    // domains as ranges of bit patterns
    struct Range { uint32_t lo, hi; bool neg; };
    std::vector<Range> ranges;
    if (is_exp) {
        ranges.push_back({0u, bits(88.5f), false});        // +0 .. 88.5
        ranges.push_back({bits(0.0f) + 1, bits(87.0f), true});  // -tiny .. -87
    } else {
        ranges.push_back({0x00800000u, 0x7F7FFFFFu, false});  // positive normal floats
    }
    std::vector<Result> res(nthreads);
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t) {
        th.emplace_back([&, t] {
            Result& r = res[t];
            for (const Range& g : ranges) {
                const uint64_t span = (uint64_t)g.hi - g.lo + 1;
                const uint64_t count = (span + stride - 1) / stride;
                for (uint64_t i = (uint64_t)t; i < count; i += (uint64_t)nthreads) {
                    uint32_t b = g.lo + (uint32_t)(i * stride);
                    const float x = g.neg ? -from_bits(b) : from_bits(b);
                    if (is_exp) check_one(x, expl((long double)x), bsg_cr::exp(x), r);
                    else check_one(x, logl((long double)x), bsg_cr::log(x), r);
                }
                // the last value of the range, always
                if (t == 0) {
                    const float x = g.neg ? -from_bits(g.hi) : from_bits(g.hi);
                    if (is_exp) check_one(x, expl((long double)x), bsg_cr::exp(x), r);
                    else check_one(x, logl((long double)x), bsg_cr::log(x), r);
                }
            }
        });
    }
    for (auto& x : th) x.join();
    Result tot;
    for (const Result& r : res) {
        tot.checked += r.checked;
        tot.misrounded += r.misrounded;
        tot.far += r.far;
        if (r.max_ulp > tot.max_ulp) tot.max_ulp = r.max_ulp;
        if (r.worst_mid > tot.worst_mid) tot.worst_mid = r.worst_mid;
    }
    std::printf("%s checked %llu misrounded %llu max_ulp %lld worst_midpoint %Lg far %llu\n",
                argv[1], (unsigned long long)tot.checked, (unsigned long long)tot.misrounded,
                (long long)tot.max_ulp, tot.worst_mid, (unsigned long long)tot.far);
    return tot.far ? 1 : 0;
}
