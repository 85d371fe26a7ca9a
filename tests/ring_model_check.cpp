// CPU model of the persistent serving kernel's tile-claim protocol
// (p3arsec_gb300/csrc/bsg_ring.h, the same code the CUDA kernel runs): one
// publisher thread plays the host, worker threads play the GPU's blocks,
// over a ring small enough that every slot is reused hundreds of times.
// Checks that every tile of every request is claimed exactly once, that
// completion is reported exactly once per request and only after all its
// tiles were done, and that nothing is left unclaimed.
//
//   ring_model_check <requests> <workers> <ring> <seed> [window]   -> prints "ok"
//
// window 1 (the default): every worker claims from the oldest request with
// unclaimed tiles; window W > 1: from the W oldest published requests, each
// worker starting at its own rotating offset (claim_window).
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <thread>
#include <vector>

#include "bsg_ring.h"

namespace {

struct HostOps {
    std::atomic<uint64_t>* taken;
    std::atomic<uint64_t>* done;
    std::atomic<uint64_t>* nt;
    uint64_t load(uint64_t s) { return taken[s].load(std::memory_order_relaxed); }
    uint64_t cas(uint64_t s, uint64_t expect, uint64_t want) {
        uint64_t seen = expect;
        taken[s].compare_exchange_strong(seen, want, std::memory_order_acq_rel);
        return seen;  // the previous value, as atomicCAS returns it
    }
    uint64_t add(uint64_t s) { return taken[s].fetch_add(1, std::memory_order_acq_rel); }
    uint64_t ntiles(uint64_t s) { return nt[s].load(std::memory_order_relaxed); }
    uint64_t done_add(uint64_t s) { return done[s].fetch_add(1, std::memory_order_acq_rel); }
    void done_reset(uint64_t s) { done[s].store(0, std::memory_order_relaxed); }
};

int fail(const char* what, uint64_t a, uint64_t b) {
    std::printf("FAIL: %s (%llu, %llu)\n", what, (unsigned long long)a, (unsigned long long)b);
    return 1;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 5 && argc != 6) return fail("usage", 0, 0);
    const uint64_t window = argc == 6 ? std::strtoull(argv[5], nullptr, 10) : 1;
    const uint64_t nreq = std::strtoull(argv[1], nullptr, 10);
    const int nworkers = std::atoi(argv[2]);
    const uint64_t ring = std::strtoull(argv[3], nullptr, 10);  // a power of two
    const uint64_t rmask = ring - 1;
    if (window < 1 || window > ring) return fail("window must be 1..ring", window, ring);
    std::mt19937_64 rng(std::strtoull(argv[4], nullptr, 10));
    std::vector<uint64_t> ntiles(nreq), first(nreq + 1, 0);
    for (uint64_t r = 0; r < nreq; ++r) {
        ntiles[r] = 1 + rng() % 40;
        first[r + 1] = first[r] + ntiles[r];
    }
    std::vector<std::atomic<uint64_t>> taken(ring), done(ring), nt(ring), flag(ring);
    for (uint64_t s = 0; s < ring; ++s) {
        taken[s] = bsg_ring::initial_word(s, ring);
        done[s] = 0;
        nt[s] = 0;
        flag[s] = 0;
    }
    std::vector<std::atomic<uint32_t>> claimed(first[nreq]);
    std::vector<std::atomic<uint32_t>> completions(nreq);
    for (auto& c : claimed) c = 0;
    for (auto& c : completions) c = 0;
    std::atomic<uint64_t> published{0}, cur{0}, completed{0};
    std::atomic<int> bad{0};

    // the host: publish request r once the slot's previous request is done
    std::thread host([&] {
        for (uint64_t r = 0; r < nreq; ++r) {
            const uint64_t s = r & rmask;
            while (r >= ring && flag[s].load(std::memory_order_acquire) != r - ring + 1)
                std::this_thread::yield();
            nt[s].store(ntiles[r], std::memory_order_relaxed);
            published.store(r + 1, std::memory_order_release);
        }
    });
    std::vector<std::thread> workers;
    for (int w = 0; w < nworkers; ++w) {
        workers.emplace_back([&, w] {
            HostOps ops{taken.data(), done.data(), nt.data()};
            std::mt19937 jitter(w);
            uint64_t rot = 0;
            while (completed.load(std::memory_order_acquire) < nreq) {
                const uint64_t r = cur.load(std::memory_order_relaxed);
                if (jitter() % 8 == 0) std::this_thread::yield();  // stale views of cur
                const uint64_t pub = published.load(std::memory_order_acquire);
                if (r >= pub) {
                    std::this_thread::yield();
                    continue;
                }
                uint64_t q = 0, tile = 0, n = 0;
                int got;
                if (window == 1) {
                    got = bsg_ring::claim(ops, r, rmask, &q, &tile, &n);
                } else if (bsg_ring::exhausted(ops, r, rmask)) {
                    got = bsg_ring::kFinished;
                } else {
                    got = bsg_ring::claim_window(ops, r, pub, rmask, window, (uint64_t)w + rot++, &q,
                                                 &tile, &n);
                }
                if (got != bsg_ring::kTile) {
                    uint64_t e = r;
                    cur.compare_exchange_strong(e, r + 1, std::memory_order_acq_rel);
                    continue;
                }
                // q is a request of the window (or a later request of one of
                // its slots), already published
                if (q < r || q >= published.load(std::memory_order_acquire)) bad = 5;
                if (window == 1 && (q - r) % ring != 0) bad = 5;
                if (q >= nreq || n != ntiles[q] || tile >= n) {
                    bad = 1;
                    continue;
                }
                if (claimed[first[q] + tile].fetch_add(1) != 0) bad = 2;  // claimed twice
                if (jitter() % 4 == 0) std::this_thread::yield();          // "pricing"
                if (bsg_ring::finish(ops, q & rmask, n)) {
                    for (uint64_t t = 0; t < n; ++t)
                        if (claimed[first[q] + t].load() != 1) bad = 3;  // done too early
                    if (completions[q].fetch_add(1) != 0) bad = 4;
                    flag[q & rmask].store(q + 1, std::memory_order_release);
                    completed.fetch_add(1, std::memory_order_acq_rel);
                }
            }
        });
    }
    host.join();
    for (auto& t : workers) t.join();
    if (bad) return fail("protocol violation", (uint64_t)bad.load(), 0);
    for (uint64_t i = 0; i < first[nreq]; ++i)
        if (claimed[i].load() != 1) return fail("tile not claimed exactly once", i, claimed[i].load());
    for (uint64_t r = 0; r < nreq; ++r)
        if (completions[r].load() != 1) return fail("completion not reported once", r, completions[r].load());
    std::printf("ok %llu requests, %llu tiles, ring %llu, %d workers\n", (unsigned long long)nreq,
                (unsigned long long)first[nreq], (unsigned long long)ring, nworkers);
    return 0;
}
