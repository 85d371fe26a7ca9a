// bsg_ring.h -- the tile-claim protocol of the persistent serving kernel,
// shared by the CUDA kernel (bsg_serve.cu) and a multi-threaded CPU model of
// it (tests/ring_model_check.cpp), so that the model checks the same code.
//
// Requests are numbered 0, 1, 2, ... and live in a ring of R slots (request
// r in slot r % R).  Each slot has a claim word and a done count:
//
//   claim word = tag (low 32 bits of r) << 32 | ntiles << 20 | tiles claimed
//
// A worker that is about to work on request r (already published; any
// published request, not only the oldest: claim_window spreads the workers
// over the oldest few):
//   * finds the slot tagged with an earlier lap: it re-arms the word for r
//     (CAS from the value it saw to tag r, ntiles of r, count 0);
//   * finds tag r: one fetch-add claims the tile numbered by the count it
//     replaced, if that count < ntiles (else every tile of r is claimed);
//   * finds a later lap: request r is finished.
// The fetch-add is blind: between reading the word and adding, the slot may
// have been re-armed for a later request r + k * R.  The add then took that
// request's tile (if its count was < ntiles) and the worker must price it:
// claim() reports the request a tile belongs to, which is not always r.
// A claimed tile is counted done after it is priced; the worker whose count
// completes the request resets the done count and reports completion, after
// which the slot may be rewritten for request r + R.
//
// Ops supplies the memory operations: load(slot), cas(slot, expected,
// desired) -> previous value, add(slot) -> previous value (fetch-add 1),
// ntiles(slot) -> the tile count of the request published in the slot,
// done_add(slot) -> previous done count (fetch-add 1), done_reset(slot).
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define BSG_RING_FN __host__ __device__ __forceinline__
#else
#define BSG_RING_FN inline
#endif

namespace bsg_ring {

constexpr uint64_t kMaxTiles = 4095;    // 12 bits
constexpr uint64_t kCountMask = 0xFFFFF;  // 20 bits of claims per lap

BSG_RING_FN uint64_t word(uint64_t r, uint64_t ntiles, uint64_t count) {
    return (uint64_t)(uint32_t)r << 32 | ntiles << 20 | count;
}
BSG_RING_FN uint32_t tag_of(uint64_t w) { return (uint32_t)(w >> 32); }
BSG_RING_FN uint64_t ntiles_of(uint64_t w) { return (w >> 20) & kMaxTiles; }
BSG_RING_FN uint64_t count_of(uint64_t w) { return w & kCountMask; }
// The word every slot starts with: armed for the lap before request `slot`.
BSG_RING_FN uint64_t initial_word(uint64_t slot, uint64_t ring) {
    return (uint64_t)(uint32_t)(slot - ring) << 32;
}

enum Claim { kTile = 0, kFinished = 1 };

// The protocol functions are templates over Ops whose members may be
// device-only (atomics): let nvcc instantiate them for the side that calls.
#if defined(__CUDACC__)
#pragma nv_exec_check_disable
#endif
// One attempt to claim a tile of published request r: kTile with *req, *tile
// and *ntiles set (*req is r, or a later request of the same slot), or
// kFinished when r has no unclaimed tile left.
template <class Ops>
BSG_RING_FN int claim(Ops& ops, uint64_t r, uint64_t rmask, uint64_t* req, uint64_t* tile,
                      uint64_t* ntiles) {
    const uint64_t slot = r & rmask;
    const uint32_t tag = (uint32_t)r;
    uint64_t w = ops.load(slot);
    for (;;) {
        const int lap = (int)(tag_of(w) - tag);
        if (lap < 0) {  // armed for an earlier lap: arm it for r
            const uint64_t want = word(r, ops.ntiles(slot), 0);
            const uint64_t seen = ops.cas(slot, w, want);
            w = (seen == w) ? want : seen;
            continue;
        }
        if (lap > 0) return kFinished;  // a later lap: r is done
        // every tile of r already claimed (counts only grow within a lap):
        // no add, so that repeated attempts on a finished request do not
        // run its count up
        if (count_of(w) >= ntiles_of(w)) return kFinished;
        const uint64_t old = ops.add(slot);
        const int lap_old = (int)(tag_of(old) - tag);
        if (count_of(old) < ntiles_of(old) && lap_old >= 0) {
            // a tile of r, or of the later request the slot was re-armed for
            *req = r + (uint64_t)(int64_t)lap_old;
            *tile = count_of(old);
            *ntiles = ntiles_of(old);
            return kTile;
        }
        if (lap_old > 0) return kFinished;  // re-armed for a later lap: r is done
        if (lap_old < 0) {  // the add hit the previous lap's (finished) word: arm it
            w = old + 1;
            continue;
        }
        return kFinished;  // every tile of r is claimed
    }
}

// True when claim word w (of request r's slot) shows no unclaimed tile of r.
BSG_RING_FN bool word_exhausted(uint64_t w, uint64_t r) {
    const int lap = (int)(tag_of(w) - (uint32_t)r);
    return lap > 0 || (lap == 0 && count_of(w) >= ntiles_of(w));
}

// True when published request r has no unclaimed tile left (one load; a
// slot not yet armed for r counts as not exhausted).
#if defined(__CUDACC__)
#pragma nv_exec_check_disable
#endif
template <class Ops>
BSG_RING_FN bool exhausted(Ops& ops, uint64_t r, uint64_t rmask) {
    return word_exhausted(ops.load(r & rmask), r);
}

// One attempt to claim a tile of one of the oldest published requests
// [r0, r0 + min(pub - r0, window)), trying them in turn from r0 + start
// (mod the window's size): requests in flight share the workers instead of
// waiting for the oldest to be fully claimed.  kTile as claim() reports it,
// or kFinished when no request of the window has an unclaimed tile.
// window <= ring size, r0 < pub.
#if defined(__CUDACC__)
#pragma nv_exec_check_disable
#endif
template <class Ops>
BSG_RING_FN int claim_window(Ops& ops, uint64_t r0, uint64_t pub, uint64_t rmask, uint64_t window,
                             uint64_t start, uint64_t* req, uint64_t* tile, uint64_t* ntiles) {
    const uint64_t w = (pub - r0 < window) ? pub - r0 : window;
    for (uint64_t k = 0; k < w; ++k)
        if (claim(ops, r0 + (start + k) % w, rmask, req, tile, ntiles) == kTile) return kTile;
    return kFinished;
}

// Counts one priced tile of the request in `slot` (ntiles tiles); true for
// the worker that completed the request, which has reset the count.
#if defined(__CUDACC__)
#pragma nv_exec_check_disable
#endif
template <class Ops>
BSG_RING_FN bool finish(Ops& ops, uint64_t slot, uint64_t ntiles) {
    if (ops.done_add(slot) + 1 != ntiles) return false;
    ops.done_reset(slot);
    return true;
}

}  // namespace bsg_ring
