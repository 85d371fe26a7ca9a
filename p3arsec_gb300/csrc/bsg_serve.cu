// bsg_serve.cu -- the request loop: continuous batching of pricing requests.
//
// Threads:
//  * callers submit requests (bsg_server_submit) into a FIFO queue;
//  * the dispatcher admits queued requests while the device pool (the
//    memory budget) and a batch slot are free, coalesces everything admitted
//    into one batch and enqueues it on the slot's stream;
//  * the completer waits (bounded, polling cudaEventQuery) for batches in
//    launch order, frees their pool ranges and completes their requests.
// Up to max_inflight batches are on the GPU at once, so requests arriving
// while a batch runs are admitted into the next one and their transfers and
// pricing overlap the running batch.
//
// Batched path, per batch: one table upload, an ingest kernel that gathers
// every request's inputs from registered (pinned) host memory into the pool,
// the persistent batch kernel over the requests' pool segments, and an
// egress kernel that writes the prices to each request's host output.  No
// per-request copy calls.  Plain path (plain = 1): one thread prices one
// request at a time with six host-to-device copies, one plain map launch and
// one device-to-host copy, and completes it itself.
#include "bsg.h"
#include "bsg_internal.h"
#include "bsg_math.cuh"
#include "bsg_ring.h"

#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <random>
#include <thread>
#include <unordered_map>
#include <vector>

#ifdef __linux__
#include <sys/prctl.h>
#endif

namespace {

constexpr uint64_t kTile = 2048;   // options per ingest/egress/batch tile: small,
                                   // so one request spreads over many SMs
constexpr uint64_t kAlign = 64;    // pool ranges start 256-byte aligned
constexpr int kThreads = 256;

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// The completer's timer slack is set to 1 us (a per-thread setting) so that
// its short sleeps between event queries end on time instead of after the
// default 50 us slack.
void set_fine_timer_slack() {
#ifdef __linux__
    prctl(PR_SET_TIMERSLACK, 1000UL, 0UL, 0UL, 0UL);
#endif
}

// One request of a batch as the ingest/egress kernels see it.  Host arrays
// are given by their device-usable addresses.
struct Desc {
    const float* src[5];
    const int32_t* ot;
    float* out;
    uint64_t off;  // pool offset in options
    uint64_t n;
    uint64_t vec;  // 1: every host array 16-byte aligned (float4 transfers)
};

__device__ __forceinline__ int find_segment(const uint64_t* pre, int m, uint64_t tile) {
    int lo = 0, hi = m - 1;
    while (lo < hi) {  // largest request whose first tile <= tile
        const int mid = (lo + hi + 1) >> 1;
        if (pre[mid] <= tile) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Host -> pool: 6 arrays of every request, tile by tile.
__global__ void __launch_bounds__(kThreads) ingest_kernel(const Desc* __restrict__ d,
                                                          const uint64_t* __restrict__ pre, int m,
                                                          uint64_t ntiles, bsg::SoA pool) {
    __shared__ int sh_q;
    float* ps = const_cast<float*>(pool.s);
    float* pk = const_cast<float*>(pool.k);
    float* pr = const_cast<float*>(pool.r);
    float* pv = const_cast<float*>(pool.v);
    float* pt = const_cast<float*>(pool.t);
    int32_t* po = const_cast<int32_t*>(pool.ot);
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        if (threadIdx.x == 0) sh_q = find_segment(pre, m, tile);
        __syncthreads();
        const Desc q = d[sh_q];
        const uint64_t b = (tile - pre[sh_q]) * kTile;
        const uint64_t e = (b + kTile < q.n) ? b + kTile : q.n;
        // float4 body when the host arrays allow it (pool offsets are 64-
        // option aligned and b is a multiple of 4), scalar rest
        const uint64_t e4 = q.vec ? b + ((e - b) & ~3ull) : b;
        for (uint64_t g = b / 4 + threadIdx.x; g < e4 / 4; g += kThreads) {
            const uint64_t o = q.off / 4 + g;
            reinterpret_cast<float4*>(ps)[o] = reinterpret_cast<const float4*>(q.src[0])[g];
            reinterpret_cast<float4*>(pk)[o] = reinterpret_cast<const float4*>(q.src[1])[g];
            reinterpret_cast<float4*>(pr)[o] = reinterpret_cast<const float4*>(q.src[2])[g];
            reinterpret_cast<float4*>(pv)[o] = reinterpret_cast<const float4*>(q.src[3])[g];
            reinterpret_cast<float4*>(pt)[o] = reinterpret_cast<const float4*>(q.src[4])[g];
            reinterpret_cast<int4*>(po)[o] = reinterpret_cast<const int4*>(q.ot)[g];
        }
        for (uint64_t i = e4 + threadIdx.x; i < e; i += kThreads) {
            const uint64_t o = q.off + i;
            ps[o] = q.src[0][i];
            pk[o] = q.src[1][i];
            pr[o] = q.src[2][i];
            pv[o] = q.src[3][i];
            pt[o] = q.src[4][i];
            po[o] = q.ot[i];
        }
        __syncthreads();
    }
}

// Pool prices -> each request's host output.
__global__ void __launch_bounds__(kThreads) egress_kernel(const Desc* __restrict__ d,
                                                          const uint64_t* __restrict__ pre, int m,
                                                          uint64_t ntiles,
                                                          const float* __restrict__ pool_out) {
    __shared__ int sh_q;
    for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        if (threadIdx.x == 0) sh_q = find_segment(pre, m, tile);
        __syncthreads();
        const Desc q = d[sh_q];
        const uint64_t b = (tile - pre[sh_q]) * kTile;
        const uint64_t e = (b + kTile < q.n) ? b + kTile : q.n;
        const uint64_t e4 = q.vec ? b + ((e - b) & ~3ull) : b;
        for (uint64_t g = b / 4 + threadIdx.x; g < e4 / 4; g += kThreads)
            reinterpret_cast<float4*>(q.out)[g] = reinterpret_cast<const float4*>(pool_out)[q.off / 4 + g];
        for (uint64_t i = e4 + threadIdx.x; i < e; i += kThreads) q.out[i] = pool_out[q.off + i];
        __syncthreads();
    }
}

// Prices options [b, min(b + kTile, n)) of request q: inputs read from the
// request's (host) arrays, prices written to its (host) output.  A thread
// issues the loads of both of its 4-option groups of a full tile before
// pricing either, so a block keeps 12 requests per thread in flight.
template <int M>
__device__ __forceinline__ void price_request_tile(const Desc& q, uint64_t b) {
    static_assert(kTile == 8 * kThreads, "two 4-option groups per thread per tile");
    const uint64_t e = (b + kTile < q.n) ? b + kTile : q.n;
    const uint64_t e4 = q.vec ? b + ((e - b) & ~3ull) : b;
    if (e4 - b == kTile) {  // a full vector tile: both groups' loads first
        const uint64_t g0 = b / 4 + threadIdx.x, g1 = g0 + kThreads;
        const float4 S0 = reinterpret_cast<const float4*>(q.src[0])[g0];
        const float4 K0 = reinterpret_cast<const float4*>(q.src[1])[g0];
        const float4 R0 = reinterpret_cast<const float4*>(q.src[2])[g0];
        const float4 V0 = reinterpret_cast<const float4*>(q.src[3])[g0];
        const float4 T0 = reinterpret_cast<const float4*>(q.src[4])[g0];
        const int4 O0 = reinterpret_cast<const int4*>(q.ot)[g0];
        const float4 S1 = reinterpret_cast<const float4*>(q.src[0])[g1];
        const float4 K1 = reinterpret_cast<const float4*>(q.src[1])[g1];
        const float4 R1 = reinterpret_cast<const float4*>(q.src[2])[g1];
        const float4 V1 = reinterpret_cast<const float4*>(q.src[3])[g1];
        const float4 T1 = reinterpret_cast<const float4*>(q.src[4])[g1];
        const int4 O1 = reinterpret_cast<const int4*>(q.ot)[g1];
        reinterpret_cast<float4*>(q.out)[g0] = bsg::price4<M>(S0, K0, R0, V0, T0, O0);
        reinterpret_cast<float4*>(q.out)[g1] = bsg::price4<M>(S1, K1, R1, V1, T1, O1);
        return;
    }
    for (uint64_t g = b / 4 + threadIdx.x; g < e4 / 4; g += kThreads) {
        const float4 S = reinterpret_cast<const float4*>(q.src[0])[g];
        const float4 K = reinterpret_cast<const float4*>(q.src[1])[g];
        const float4 R = reinterpret_cast<const float4*>(q.src[2])[g];
        const float4 V = reinterpret_cast<const float4*>(q.src[3])[g];
        const float4 T = reinterpret_cast<const float4*>(q.src[4])[g];
        const int4 O = reinterpret_cast<const int4*>(q.ot)[g];
        reinterpret_cast<float4*>(q.out)[g] = bsg::price4<M>(S, K, R, V, T, O);
    }
    for (uint64_t i = e4 + threadIdx.x; i < e; i += kThreads)
        q.out[i] = bsg::price<M>(q.src[0][i], q.src[1][i], q.src[2][i], q.src[3][i],
                                 q.src[4][i], q.ot[i]);
}

// Fused path: one kernel per batch reads each request's inputs from host
// memory, prices them and writes the prices back to the request's host
// output.  Tiles come from a per-slot counter that only grows: this launch's
// tiles are [base, base + ntiles) of it, and every block ends with exactly
// one failing increment, so the next launch's base is base + ntiles + grid
// (no reset between batches).
template <int M>
__device__ __forceinline__ void fused_tiles(const Desc* __restrict__ d,
                                            const uint64_t* __restrict__ pre, int m,
                                            uint64_t ntiles, unsigned long long* counter,
                                            unsigned long long base) {
    __shared__ int sh_q, sh_done;
    __shared__ uint64_t sh_tile;
    for (;;) {
        if (threadIdx.x == 0) {
            const unsigned long long t = atomicAdd(counter, 1ull) - base;
            sh_done = t >= ntiles;
            if (!sh_done) {
                sh_tile = t;
                sh_q = find_segment(pre, m, t);
            }
        }
        __syncthreads();
        if (sh_done) break;
        const int qi = sh_q;
        const uint64_t tile = sh_tile;
        __syncthreads();
        price_request_tile<M>(d[qi], (tile - pre[qi]) * kTile);
    }
}

// Table in device memory (copied there before the launch).
template <int M>
__global__ void __launch_bounds__(kThreads) serve_fused_kernel(const Desc* __restrict__ d,
                                                               const uint64_t* __restrict__ pre,
                                                               int m, uint64_t ntiles,
                                                               unsigned long long* counter,
                                                               unsigned long long base) {
    fused_tiles<M>(d, pre, m, ntiles, counter, base);
}

// Batches of up to kInline requests carry their table in the kernel's
// parameters (__grid_constant__: read in place, no copy before the launch).
constexpr int kInline = 24;
struct InlineTable {
    Desc d[kInline];
    uint64_t pre[kInline + 1];
};
static_assert(sizeof(InlineTable) <= 4000, "kernel parameter space");

template <int M>
__global__ void __launch_bounds__(kThreads) serve_fused_inline_kernel(
    const __grid_constant__ InlineTable tab, int m, uint64_t ntiles,
    unsigned long long* counter, unsigned long long base) {
    fused_tiles<M>(tab.d, tab.pre, m, ntiles, counter, base);
}

cudaError_t launch_fused(int mode, unsigned grid, cudaStream_t st, const Desc* d,
                         const uint64_t* pre, int m, uint64_t ntiles,
                         unsigned long long* counter, unsigned long long base) {
    switch (mode) {
        case bsg::MODE_FAST:
            serve_fused_kernel<bsg::MODE_FAST><<<grid, kThreads, 0, st>>>(d, pre, m, ntiles, counter, base);
            break;
        case bsg::MODE_SFU_REF:
            serve_fused_kernel<bsg::MODE_SFU_REF><<<grid, kThreads, 0, st>>>(d, pre, m, ntiles, counter, base);
            break;
        default:
            serve_fused_kernel<bsg::MODE_LIBM_REF><<<grid, kThreads, 0, st>>>(d, pre, m, ntiles, counter, base);
            break;
    }
    return cudaGetLastError();
}

cudaError_t launch_fused_inline(int mode, unsigned grid, cudaStream_t st, const InlineTable& tab,
                                int m, uint64_t ntiles, unsigned long long* counter,
                                unsigned long long base) {
    switch (mode) {
        case bsg::MODE_FAST:
            serve_fused_inline_kernel<bsg::MODE_FAST><<<grid, kThreads, 0, st>>>(tab, m, ntiles, counter, base);
            break;
        case bsg::MODE_SFU_REF:
            serve_fused_inline_kernel<bsg::MODE_SFU_REF><<<grid, kThreads, 0, st>>>(tab, m, ntiles, counter, base);
            break;
        default:
            serve_fused_inline_kernel<bsg::MODE_LIBM_REF><<<grid, kThreads, 0, st>>>(tab, m, ntiles, counter, base);
            break;
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Persistent path: one kernel keeps running while requests arrive.  The host
// writes each request into a ring of entries in pinned host memory (read by
// the GPU over NVLink-C2C) and raises `published`; the blocks take tiles of
// the oldest request with unclaimed tiles, price them, and the block that
// finishes a request's last tile sets the entry's completion flag, which the
// host polls.  No launch, table copy or event per request.
//
// Tile claims and done counts live in device memory (GPU-scope atomics; one
// word of each per ring slot, reused lap after lap).  Claim word = tag (low 32
// bits of the request's sequence number) << 32 | ntiles << 20 | tiles
// claimed.  A block that sees its request's tag claims with one add and
// decodes the value it replaced (count < ntiles: a tile); a slot still
// tagged with the previous lap is re-armed for the request with a CAS, its
// tile count read from the published entry; a slot tagged with a later lap
// means the request is finished.  The only wait is a block finding no
// published work: bounded by idle_ns of GPU time (and the host's stop
// flag), after which the block exits; the host relaunches the kernel when
// work arrives and no kernel is running.
constexpr uint64_t kMaxRequestTiles = bsg_ring::kMaxTiles;  // 12 bits of the claim word
// Requests the persistent kernel's blocks share at once (bsg_ring::claim_window);
// 1 = the oldest request's tiles first.
constexpr unsigned long long kDefaultWindow = 1;
constexpr unsigned long long kMaxWindow = 16;  // claim words a block loads at once
constexpr int kDescCache = 4;                  // request descriptors a block keeps

struct alignas(128) PEntry {
    unsigned long long flag;    // seq + 1 once every tile is priced (GPU writes)
    unsigned long long seq;     // request sequence number
    unsigned long long ntiles;
    Desc d;
};

struct alignas(64) PCtl {
    unsigned long long published;   // requests 0 .. published-1 are in the ring
    unsigned long long pad[7];
    unsigned int stop;              // 1: blocks exit at their next idle check
};

__device__ __forceinline__ unsigned long long ld_acquire_sys(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned ld_relaxed_sys_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.relaxed.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long ld_acquire_gpu(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned long long ld_relaxed_gpu(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned atom_add_acq_rel_gpu(unsigned* p, unsigned v) {
    unsigned old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ void st_release_sys(unsigned long long* p, unsigned long long v) {
    asm volatile("st.release.sys.global.u64 [%0], %1;" :: "l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// The claim protocol's memory operations on the device (bsg_ring.h): claim
// words and done counts in device memory, tile counts from the published
// entries in host memory.
struct DeviceRingOps {
    unsigned long long* taken;
    unsigned* done;
    const PEntry* ring;
    __device__ uint64_t load(uint64_t s) { return ld_relaxed_gpu(taken + s); }
    __device__ uint64_t cas(uint64_t s, uint64_t expect, uint64_t want) {
        return atomicCAS(taken + s, (unsigned long long)expect, (unsigned long long)want);
    }
    __device__ uint64_t add(uint64_t s) { return atomicAdd(taken + s, 1ull); }
    __device__ uint64_t ntiles(uint64_t s) { return ring[s].ntiles; }
    __device__ uint64_t done_add(uint64_t s) { return atom_add_acq_rel_gpu(done + s, 1u); }
    __device__ void done_reset(uint64_t s) { done[s] = 0u; }
};

template <int M>
__global__ void __launch_bounds__(kThreads) serve_persistent_kernel(
    PEntry* ring, unsigned long long rmask, const PCtl* ctl, unsigned long long* cur,
    unsigned long long* taken, unsigned* done, unsigned long long idle_ns,
    unsigned long long window) {
    __shared__ Desc sh_d;
    __shared__ unsigned long long sh_b, sh_seq, sh_nt;
    __shared__ int sh_ok;
    __shared__ Desc sh_cache[kDescCache];
    __shared__ unsigned long long sh_cseq[kDescCache];
    if (threadIdx.x < kDescCache) sh_cseq[threadIdx.x] = ~0ull;
    __syncthreads();
    // thread 0's view of `published` (re-read from host memory only when the
    // ring looks drained) and the request whose descriptor sh_d holds.  While
    // idle, only the first kScouts blocks poll host memory; they copy what
    // they see into a device word (cur[1]) that the other blocks poll in L2,
    // so every block notices new work within about a microsecond without
    // hundreds of blocks reading across the link.
    constexpr unsigned kScouts = 8;
    const bool scout = blockIdx.x < kScouts;
    unsigned long long* pub_dev = cur + 1;
    unsigned long long pub = 0, d_seq = ~0ull, rot = 0, cnext = 0;
    for (;;) {
        if (threadIdx.x == 0) {
            sh_ok = 0;
            unsigned backoff = 64, polls = 0;
            unsigned long long t0 = global_ns();
            while (ld_relaxed_sys_u32(&ctl->stop) == 0) {
                const unsigned long long r = ld_relaxed_gpu(cur);
                if (r >= pub) {
                    // (a non-scout also reads the host's count itself every
                    // 32nd poll, in case every scout is busy pricing)
                    if (scout || (++polls & 31) == 0) {
                        pub = ld_acquire_sys(&ctl->published);
                        if (pub > r) atomicMax(pub_dev, pub);
                    } else if (ld_acquire_gpu(pub_dev) > r) {
                        pub = ld_acquire_sys(&ctl->published);  // see the entries too
                    }
                }
                if (r >= pub) {  // nothing published
                    if (global_ns() - t0 > idle_ns) break;  // bounded idle wait
                    __nanosleep(backoff);
                    if (backoff < 1024) backoff *= 2;
                    continue;
                }
                DeviceRingOps ops{taken, done, ring};
                uint64_t q = 0, c = 0, nt = 0;
                int got = bsg_ring::kFinished;
                if (window <= 1) {
                    // the oldest request's tiles first, in order of arrival
                    got = bsg_ring::claim(ops, r, rmask, &q, &c, &nt);
                } else {
                    // a tile of one of the w oldest published requests, so
                    // that requests in flight share the blocks: their claim
                    // words loaded together (one round trip), the cursor
                    // moved past the leading finished ones, then the live
                    // ones tried from this block's rotating offset (each
                    // claim as bsg_ring::claim_window makes it)
                    const uint64_t w = (pub - r < window) ? pub - r : window;
                    uint64_t wv[kMaxWindow];
#pragma unroll
                    for (int k = 0; k < (int)kMaxWindow; ++k)
                        if ((uint64_t)k < w) wv[k] = ops.load((r + k) & rmask);
                    uint64_t lead = 0;
                    while (lead < w && bsg_ring::word_exhausted(wv[lead], r + lead)) ++lead;
                    if (lead > 0) {
                        atomicCAS(cur, r, r + lead);
                        if (lead == w) {
                            t0 = global_ns();
                            backoff = 64;
                            continue;
                        }
                    }
                    uint64_t i = (blockIdx.x + rot++) % w;
                    for (uint64_t k = 0; k < w && got != bsg_ring::kTile; ++k, i = (i + 1 == w) ? 0 : i + 1)
                        if (!bsg_ring::word_exhausted(wv[i], r + i))
                            got = bsg_ring::claim(ops, r + i, rmask, &q, &c, &nt);
                    if (got != bsg_ring::kTile) continue;  // claimed meanwhile: look again
                }
                if (got == bsg_ring::kTile) {
                    // a tile of q: r, or a later request of the same slot,
                    // which another block armed after seeing it published;
                    // see that publication here too before reading q's entry
                    // (bounded: it happened before the arming)
                    for (int i = 0; q >= pub && i < (1 << 20); ++i)
                        pub = ld_acquire_sys(&ctl->published);
                    const unsigned long long slot = q & rmask;
                    if (d_seq != q) {
                        // the descriptors of the last kDescCache requests
                        // this block priced stay in shared memory: a block
                        // moving between requests reads each from host
                        // memory once
                        int hit = -1;
                        for (int k = 0; k < kDescCache; ++k)
                            if (sh_cseq[k] == q) hit = k;
                        if (hit < 0) {
                            hit = (int)(cnext++ % kDescCache);
                            sh_cache[hit] = ring[slot].d;
                            sh_cseq[hit] = q;
                        }
                        sh_d = sh_cache[hit];
                        d_seq = q;
                    }
                    sh_b = c * kTile;
                    sh_seq = q;
                    sh_nt = nt;
                    sh_ok = 1;
                    break;
                }
                atomicCAS(cur, r, r + 1);  // r (the window) has no unclaimed tile: move on
                t0 = global_ns();
                backoff = 64;
            }
        }
        __syncthreads();
        if (!sh_ok) break;
        const Desc q = sh_d;
        price_request_tile<M>(q, sh_b);
        __threadfence_system();  // this thread's prices reach host memory first
        __syncthreads();
        if (threadIdx.x == 0) {
            // the request's last tile: every block's prices are in host
            // memory (each fenced before its count); the count is re-armed
            DeviceRingOps ops{taken, done, ring};
            const unsigned long long slot = sh_seq & rmask;
            if (bsg_ring::finish(ops, slot, sh_nt)) st_release_sys(&ring[slot].flag, sh_seq + 1ull);
        }
    }
}

cudaError_t launch_persistent(int mode, unsigned grid, cudaStream_t st, PEntry* ring,
                              unsigned long long rmask, const PCtl* ctl, unsigned long long* cur,
                              unsigned long long* taken, unsigned* done,
                              unsigned long long idle_ns, unsigned long long window) {
    switch (mode) {
        case bsg::MODE_FAST:
            serve_persistent_kernel<bsg::MODE_FAST><<<grid, kThreads, 0, st>>>(ring, rmask, ctl, cur, taken, done, idle_ns, window);
            break;
        case bsg::MODE_SFU_REF:
            serve_persistent_kernel<bsg::MODE_SFU_REF><<<grid, kThreads, 0, st>>>(ring, rmask, ctl, cur, taken, done, idle_ns, window);
            break;
        default:
            serve_persistent_kernel<bsg::MODE_LIBM_REF><<<grid, kThreads, 0, st>>>(ring, rmask, ctl, cur, taken, done, idle_ns, window);
            break;
    }
    return cudaGetLastError();
}

enum State { Q_QUEUED, Q_ADMITTED, Q_DONE };

struct Request {
    uint64_t id;
    bsg_request r;
    uint64_t span;  // pool options held (n rounded up to kAlign)
    uint64_t off;
    double t_ref;   // latency reference: submit time or scheduled arrival
    double t_done;
    State state;
    int status;
    bool auto_release;
    double* lat_slot;
    Desc desc;
    uint64_t seq = 0, ntiles = 0;  // persistent path: ring sequence number, tiles
    double t_pub = 0;              // persistent path: publication time
};

struct Slot {
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    char* h_tab = nullptr;  // pinned table block
    char* d_tab = nullptr;  // device table block
    unsigned long long* d_cursor = nullptr;
    unsigned long long fused_base = 0;  // next launch's base on the fused counter
    std::vector<Request*> reqs;
    bool busy = false;
};

struct HostRange {
    uintptr_t b, e;
    intptr_t delta;  // device address = host address + delta
    bool owned;      // registered by us (unregister at destroy)
};

// The driver's record of the CUDA allocation or registration containing p
// (cuPointerGetAttribute RANGE_START_ADDR / RANGE_SIZE), resolved at run time.
typedef CUresult (*PtrAttrFn)(void*, CUpointer_attribute, CUdeviceptr);

bool cuda_range(const void* p, uintptr_t* b, size_t* sz) {
    static PtrAttrFn fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuPointerGetAttribute", &f, 12000,
                                             cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            f = nullptr;
        }
        return reinterpret_cast<PtrAttrFn>(f);
    }();
    if (!fn) return false;
    CUdeviceptr start = 0;
    size_t size = 0;
    if (fn(&start, CU_POINTER_ATTRIBUTE_RANGE_START_ADDR, (CUdeviceptr)p) != CUDA_SUCCESS ||
        fn(&size, CU_POINTER_ATTRIBUTE_RANGE_SIZE, (CUdeviceptr)p) != CUDA_SUCCESS)
        return false;
    *b = (uintptr_t)start;
    *sz = size;
    return true;
}

size_t table_bytes(int cap) {
    return (size_t)cap * sizeof(Desc) + (3 * (size_t)cap + 1) * sizeof(uint64_t);
}

}  // namespace

constexpr uint64_t kRing = 4096;                 // persistent ring entries
constexpr unsigned long long kIdleNs = 5000000;  // a block's idle bound: 5 ms
constexpr double kPollWindow = 5e-3;             // completer polls this long after work

struct bsg_server {
    bsg_server_config cfg{};
    int device = 0, sm_count = 0, batch_grid = 1, mode = 0, max_req = 4096;
    double batch_timeout = 30.0;
    char* d_pool = nullptr;
    // persistent path (cfg.fused == 2)
    bool persistent = false, broken = false;
    PEntry* ring_h = nullptr;   // pinned host ring, and the GPU's address of it
    PEntry* ring_d = nullptr;
    PCtl* ctl_h = nullptr;
    PCtl* ctl_d = nullptr;
    // device words: [0] the oldest request that may have unclaimed tiles,
    // [1] the scouts' copy of `published` (see serve_persistent_kernel)
    unsigned long long* d_cur = nullptr;
    unsigned long long* d_taken = nullptr;  // per ring slot: claim word
    unsigned* d_done = nullptr;             // per ring slot: tiles priced
    cudaStream_t pst = nullptr;
    cudaEvent_t pev = nullptr;            // recorded after each launch of the kernel
    unsigned pgrid = 1;
    unsigned long long pwindow = 1;       // requests the blocks share (claim_window)
    uint64_t next_seq = 0;
    std::deque<Request*> pinflight;       // published, not complete, in sequence order
    uint64_t cap = 0;  // options
    bsg::SoA pool{};
    std::map<uint64_t, uint64_t> free_list;  // start -> length (options)
    std::vector<Slot> slots;
    std::vector<HostRange> hosts;
    std::mutex mu;
    std::condition_variable cv_disp, cv_comp, cv_done;
    std::deque<Request*> queue;
    std::deque<int> inflight;
    std::unordered_map<uint64_t, Request*> reqs;
    std::thread disp, comp;
    bool stop = false, paused = false;
    uint64_t next_id = 1, free_gen = 0;
    bsg_server_stats st{};

    // ------------------------------------------------------------ pool
    bool pool_alloc(uint64_t span, uint64_t* off) {
        for (auto it = free_list.begin(); it != free_list.end(); ++it) {
            if (it->second >= span) {
                *off = it->first;
                const uint64_t rest = it->second - span;
                const uint64_t start = it->first + span;
                free_list.erase(it);
                if (rest) free_list[start] = rest;
                return true;
            }
        }
        return false;
    }
    void pool_free(uint64_t off, uint64_t span) {
        auto it = free_list.emplace(off, span).first;
        auto nx = std::next(it);
        if (nx != free_list.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_list.erase(nx);
        }
        if (it != free_list.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_list.erase(it);
            }
        }
    }

    const HostRange* host_range(const void* p, size_t bytes) const {
        const uintptr_t a = reinterpret_cast<uintptr_t>(p);
        for (const auto& h : hosts)
            if (a >= h.b && a + bytes <= h.e && a + bytes >= a) return &h;
        return nullptr;
    }

    int free_slot() const {
        for (size_t i = 0; i < slots.size(); ++i)
            if (!slots[i].busy) return (int)i;
        return -1;
    }

    // --------------------------------------------------------- enqueue
    int enqueue_batched(Slot& sl) {
        bsg::NvtxRange nvtx_("bsg_server batch");
        const int m = (int)sl.reqs.size();
        Desc* hd = reinterpret_cast<Desc*>(sl.h_tab);
        uint64_t* hoff = reinterpret_cast<uint64_t*>(sl.h_tab + (size_t)m * sizeof(Desc));
        uint64_t* hlen = hoff + m;
        uint64_t* hpre = hlen + m;
        uint64_t acc = 0;
        for (int i = 0; i < m; ++i) {
            const Request* q = sl.reqs[i];
            hd[i] = q->desc;
            hoff[i] = q->off;
            hlen[i] = q->r.n;
            hpre[i] = acc;
            acc += (q->r.n + kTile - 1) / kTile;
        }
        hpre[m] = acc;
        const uint64_t ntiles = acc;
        const unsigned grid = (unsigned)std::min<uint64_t>(ntiles, (uint64_t)sm_count * 8);
        if (cfg.fused && m <= kInline) {
            // the table travels in the launch's parameters: no copy
            InlineTable tab;
            for (int i = 0; i < m; ++i) {
                tab.d[i] = hd[i];
                tab.pre[i] = hpre[i];
            }
            tab.pre[m] = hpre[m];
            unsigned long long* ctr = sl.d_cursor + 1;
            if (launch_fused_inline(mode, grid, sl.st, tab, m, ntiles, ctr, sl.fused_base) != cudaSuccess)
                return BSG_ERR_CUDA;
            sl.fused_base += ntiles + grid;
            if (cudaEventRecord(sl.ev, sl.st) != cudaSuccess) return BSG_ERR_CUDA;
            return BSG_OK;
        }
        const size_t bytes = (size_t)m * sizeof(Desc) + (3 * (size_t)m + 1) * sizeof(uint64_t);
        if (cudaMemcpyAsync(sl.d_tab, sl.h_tab, bytes, cudaMemcpyHostToDevice, sl.st) != cudaSuccess)
            return BSG_ERR_CUDA;
        const Desc* dd = reinterpret_cast<const Desc*>(sl.d_tab);
        const uint64_t* doff = reinterpret_cast<const uint64_t*>(sl.d_tab + (size_t)m * sizeof(Desc));
        const uint64_t* dlen = doff + m;
        const uint64_t* dpre = dlen + m;
        if (cfg.fused) {
            // counter lives after the batch kernel's cursor word
            unsigned long long* ctr = sl.d_cursor + 1;
            if (launch_fused(mode, grid, sl.st, dd, dpre, m, ntiles, ctr, sl.fused_base) != cudaSuccess)
                return BSG_ERR_CUDA;
            sl.fused_base += ntiles + grid;
            if (cudaEventRecord(sl.ev, sl.st) != cudaSuccess) return BSG_ERR_CUDA;
            return BSG_OK;
        }
        ingest_kernel<<<grid, kThreads, 0, sl.st>>>(dd, dpre, m, ntiles, pool);
        if (cudaGetLastError() != cudaSuccess) return BSG_ERR_CUDA;
        if (cudaMemsetAsync(sl.d_cursor, 0, sizeof(unsigned long long), sl.st) != cudaSuccess)
            return BSG_ERR_CUDA;
        if (bsg::launch_batch(pool, doff, dlen, dpre, nullptr, m, ntiles, kTile, sl.d_cursor, mode,
                              batch_grid, 0, sl.st) != cudaSuccess)
            return BSG_ERR_CUDA;
        egress_kernel<<<grid, kThreads, 0, sl.st>>>(dd, dpre, m, ntiles, pool.out);
        if (cudaGetLastError() != cudaSuccess) return BSG_ERR_CUDA;
        if (cudaEventRecord(sl.ev, sl.st) != cudaSuccess) return BSG_ERR_CUDA;
        return BSG_OK;
    }

    int enqueue_plain(Slot& sl) {
        bsg::NvtxRange nvtx_("bsg_server plain request");
        const Request* q = sl.reqs[0];
        const uint64_t o = q->off;
        const size_t b = q->r.n * 4;
        float* ps = const_cast<float*>(pool.s) + o;
        float* pk = const_cast<float*>(pool.k) + o;
        float* pr = const_cast<float*>(pool.r) + o;
        float* pv = const_cast<float*>(pool.v) + o;
        float* pt = const_cast<float*>(pool.t) + o;
        int32_t* po = const_cast<int32_t*>(pool.ot) + o;
        if (cudaMemcpyAsync(ps, q->r.sptprice, b, cudaMemcpyHostToDevice, sl.st) ||
            cudaMemcpyAsync(pk, q->r.strike, b, cudaMemcpyHostToDevice, sl.st) ||
            cudaMemcpyAsync(pr, q->r.rate, b, cudaMemcpyHostToDevice, sl.st) ||
            cudaMemcpyAsync(pv, q->r.volatility, b, cudaMemcpyHostToDevice, sl.st) ||
            cudaMemcpyAsync(pt, q->r.otime, b, cudaMemcpyHostToDevice, sl.st) ||
            cudaMemcpyAsync(po, q->r.otype, b, cudaMemcpyHostToDevice, sl.st))
            return BSG_ERR_CUDA;
        bsg::SoA a{ps, pk, pr, pv, pt, po, pool.out + o};
        const bsg::MapCfg cfg{1, 256, 0, 0, 0};
        if (bsg::launch_map(a, (int64_t)q->r.n, mode, cfg, sm_count, sl.st) != cudaSuccess)
            return BSG_ERR_CUDA;
        if (cudaMemcpyAsync(q->r.prices, pool.out + o, b, cudaMemcpyDeviceToHost, sl.st) ||
            cudaEventRecord(sl.ev, sl.st))
            return BSG_ERR_CUDA;
        return BSG_OK;
    }

    void complete(Request* q, int status, double t, bool free_range) {
        q->status = status;
        q->t_done = t;
        q->state = Q_DONE;
        if (free_range) pool_free(q->off, q->span);
        if (status == BSG_OK) {
            st.completed++;
            st.options_priced += q->r.n;
        } else if (status == BSG_ERR_CANCELLED) {
            st.cancelled++;
        } else {
            st.failed++;
        }
        if (q->auto_release) {
            if (q->lat_slot) *q->lat_slot = (status == BSG_OK) ? t - q->t_ref : NAN;
            reqs.erase(q->id);
            delete q;
        }
    }

    // ------------------------------------------------- persistent path
    // Launches the persistent kernel unless one is running.  Only the
    // completer thread calls it, without holding mu, so that a slow driver
    // call never blocks submitting threads.
    int ensure_kernel(bool* launched) {
        *launched = false;
        const cudaError_t q = cudaEventQuery(pev);
        if (q == cudaErrorNotReady) return BSG_OK;
        if (q != cudaSuccess) {
            cudaGetLastError();
            return BSG_ERR_CUDA;
        }
        // callers include submitting threads: launch on the server's device
        int prev = device;
        cudaGetDevice(&prev);
        if (prev != device) cudaSetDevice(device);
        const bool ok = launch_persistent(mode, pgrid, pst, ring_d, kRing - 1, ctl_d, d_cur,
                                          d_taken, d_done, kIdleNs,
                                          std::min<unsigned long long>(pwindow, kMaxWindow)) == cudaSuccess &&
                        cudaEventRecord(pev, pst) == cudaSuccess;
        if (prev != device) cudaSetDevice(prev);
        if (!ok) {
            cudaGetLastError();
            return BSG_ERR_CUDA;
        }
        *launched = true;
        return BSG_OK;
    }

    // Admits request q (pool range `off`), writes it into its ring entry and
    // publishes it (caller holds mu; the entry's previous request,
    // seq - kRing, is complete).
    void publish(Request* q, uint64_t off) {
        q->off = off;
        q->state = Q_ADMITTED;
        q->desc.off = off;
        q->desc.n = q->r.n;
        q->seq = next_seq++;
        q->ntiles = (q->r.n + kTile - 1) / kTile;
        PEntry* e = ring_h + (q->seq & (kRing - 1));
        e->d = q->desc;
        e->ntiles = q->ntiles;
        e->seq = q->seq;
        __atomic_store_n(&ctl_h->published, next_seq, __ATOMIC_RELEASE);
        q->t_pub = now_s();
        pinflight.push_back(q);
        st.batches++;
    }

    // Whether request q can be published now (caller holds mu); on success
    // its pool range is taken.
    bool can_publish(const Request* q, uint64_t* off) {
        const uint64_t floor = pinflight.empty() ? next_seq : pinflight.front()->seq;
        return next_seq < floor + kRing && pool_alloc(q->span, off);
    }

    void dispatcher_persistent() {
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            cv_disp.wait(lk, [&] { return stop || (!paused && !queue.empty()); });
            if (stop) break;
            bool published = false;
            while (!paused && !queue.empty()) {
                Request* q = queue.front();
                if (broken) {
                    queue.pop_front();
                    complete(q, BSG_ERR_STATE, now_s(), false);
                    cv_done.notify_all();
                    continue;
                }
                uint64_t off;
                if (!can_publish(q, &off)) break;  // wait for room
                queue.pop_front();
                publish(q, off);
                published = true;
            }
            if (published) {
                cv_comp.notify_one();  // the completer (re)launches the kernel
            } else if (!queue.empty() && !paused) {
                const uint64_t g0 = free_gen;  // wait for a completion to free room
                cv_disp.wait(lk, [&] { return stop || free_gen != g0 || paused; });
            }
        }
    }

    // Polls the completion flags of published requests (any order), every
    // few microseconds while any is outstanding, and launches the kernel
    // whenever requests are outstanding and none is running (first request,
    // or the kernel exited at its idle bound).  A request older
    // than batch_timeout fails with BSG_ERR_TIMEOUT and the server turns
    // broken: its entry may still be written by the GPU, so nothing is reused.
    void completer_persistent() {
        set_fine_timer_slack();
        std::unique_lock<std::mutex> lk(mu);
        double last_busy = now_s();
        for (;;) {
            // for a while after the last request, keep polling instead of
            // sleeping on the condition variable: a thread woken from it
            // starts tens of microseconds late, the poll within a few
            while (!stop && pinflight.empty() && now_s() - last_busy < kPollWindow) {
                lk.unlock();
                std::this_thread::sleep_for(std::chrono::microseconds(2));
                lk.lock();
            }
            cv_comp.wait(lk, [&] { return stop || !pinflight.empty(); });
            last_busy = now_s();
            if (pinflight.empty()) {
                if (stop) break;
                continue;
            }
            if (!broken) {
                bool launched = false;
                lk.unlock();
                const int krc = ensure_kernel(&launched);
                lk.lock();
                if (krc != BSG_OK) broken = true;
                if (launched) st.kernel_launches++;
            }
            const double t = now_s();
            bool freed = false;
            for (auto it = pinflight.begin(); it != pinflight.end();) {
                Request* q = *it;
                const PEntry* e = ring_h + (q->seq & (kRing - 1));
                if (__atomic_load_n(&e->flag, __ATOMIC_ACQUIRE) == q->seq + 1) {
                    complete(q, BSG_OK, t, true);
                    it = pinflight.erase(it);
                    freed = true;
                } else if (t - q->t_pub > batch_timeout) {
                    broken = true;
                    complete(q, BSG_ERR_TIMEOUT, t, false);
                    it = pinflight.erase(it);
                } else {
                    ++it;
                }
            }
            if (freed) {
                free_gen++;
                cv_done.notify_all();
                cv_disp.notify_one();
            }
            lk.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(2));
            lk.lock();
        }
    }

    // ------------------------------------------------------- plain path
    // One thread takes the requests in FIFO order and prices each in turn:
    // six copies, one plain launch, one copy back, then it polls the
    // request's event and completes it itself.  Between requests it polls
    // the queue for a while (as the persistent path's completer does), so
    // neither a new request nor a finished one waits for a thread to wake
    // from a condition variable: the baseline pays for its per-request
    // copies and launch, not for thread hand-offs.
    void dispatcher_plain() {
        set_fine_timer_slack();
        Slot& sl = slots[0];
        std::unique_lock<std::mutex> lk(mu);
        double last_busy = now_s();
        bool stuck = false;  // a request overran batch_timeout: its range stays held
        for (;;) {
            while (!stop && (stuck || paused || queue.empty()) &&
                   now_s() - last_busy < kPollWindow) {
                lk.unlock();
                std::this_thread::sleep_for(std::chrono::microseconds(2));
                lk.lock();
            }
            cv_disp.wait(lk, [&] { return stop || (!stuck && !paused && !queue.empty()); });
            if (stop) break;
            Request* q = queue.front();
            uint64_t off;
            if (!pool_alloc(q->span, &off)) {  // only one request holds the pool
                queue.pop_front();
                complete(q, BSG_ERR_BUDGET, now_s(), false);
                cv_done.notify_all();
                continue;
            }
            queue.pop_front();
            q->off = off;
            q->state = Q_ADMITTED;
            sl.reqs.assign(1, q);
            sl.busy = true;
            st.batches++;
            st.max_batch_requests_seen = std::max<uint64_t>(st.max_batch_requests_seen, 1);
            inflight.push_back(0);
            lk.unlock();
            int rc = enqueue_plain(sl);
            bool release = true;
            if (rc == BSG_OK) {
                rc = wait_event(sl.ev);
                release = rc != BSG_ERR_TIMEOUT;
            } else {
                // copies or the launch may already be enqueued: drain first
                cudaGetLastError();
                release = cudaStreamSynchronize(sl.st) == cudaSuccess;
            }
            const double t = now_s();
            lk.lock();
            inflight.pop_front();
            if (rc == BSG_OK) st.kernel_launches++;
            complete(q, rc, t, release);
            sl.reqs.clear();
            if (release) sl.busy = false;
            else stuck = true;
            free_gen++;
            cv_done.notify_all();
            last_busy = now_s();
        }
    }

    // ------------------------------------------------------- dispatcher
    void dispatcher() {
        cudaSetDevice(device);
        if (persistent) {
            dispatcher_persistent();
            return;
        }
        if (cfg.plain) {
            dispatcher_plain();
            return;
        }
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            cv_disp.wait(lk, [&] { return stop || (!paused && !queue.empty() && free_slot() >= 0); });
            if (stop) break;
            const int si = free_slot();
            Slot& sl = slots[si];
            sl.reqs.clear();
            uint64_t opts = 0;
            const int limit = cfg.plain ? 1 : max_req;
            while (!queue.empty() && (int)sl.reqs.size() < limit) {
                Request* q = queue.front();
                if (cfg.max_batch_options && !sl.reqs.empty() &&
                    opts + q->r.n > cfg.max_batch_options)
                    break;
                uint64_t off;
                if (!pool_alloc(q->span, &off)) break;  // FIFO: wait for memory
                q->off = off;
                q->state = Q_ADMITTED;
                Desc& d = q->desc;
                d.off = off;
                d.n = q->r.n;
                queue.pop_front();
                sl.reqs.push_back(q);
                opts += q->r.n;
            }
            if (sl.reqs.empty()) {
                const uint64_t g0 = free_gen;
                cv_disp.wait(lk, [&] { return stop || free_gen != g0; });
                continue;
            }
            sl.busy = true;
            st.batches++;
            st.max_batch_requests_seen = std::max<uint64_t>(st.max_batch_requests_seen, sl.reqs.size());
            lk.unlock();
            const int rc = cfg.plain ? enqueue_plain(sl) : enqueue_batched(sl);
            lk.lock();
            if (rc != BSG_OK) {
                cudaGetLastError();
                // work already enqueued may still run: keep the ranges and
                // the slot until the stream drains, then fail the requests
                lk.unlock();
                const bool drained = cudaStreamSynchronize(sl.st) == cudaSuccess;
                lk.lock();
                const double t = now_s();
                for (Request* q : sl.reqs) complete(q, rc, t, drained);
                sl.reqs.clear();
                sl.busy = !drained;
                free_gen++;
                cv_done.notify_all();
                continue;
            }
            st.kernel_launches += (cfg.plain || cfg.fused) ? 1 : 3;
            inflight.push_back(si);
            cv_comp.notify_one();
        }
    }

    // Bounded wait for one batch: cudaEventQuery, a few back to back, then
    // with 5 us sleeps (fine timer slack: see set_fine_timer_slack).
    int wait_event(cudaEvent_t ev) {
        const double t_end = now_s() + batch_timeout;
        int spins = 0;
        for (;;) {
            const cudaError_t e = cudaEventQuery(ev);
            if (e == cudaSuccess) return BSG_OK;
            if (e != cudaErrorNotReady) {
                cudaGetLastError();
                return BSG_ERR_CUDA;
            }
            if (now_s() > t_end) return BSG_ERR_TIMEOUT;
            if (++spins > 16) std::this_thread::sleep_for(std::chrono::microseconds(5));
        }
    }

    // -------------------------------------------------------- completer
    void completer() {
        cudaSetDevice(device);
        if (persistent) {
            completer_persistent();
            return;
        }
        if (cfg.plain) return;  // the plain path's dispatcher completes its requests
        set_fine_timer_slack();
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            cv_comp.wait(lk, [&] { return stop || !inflight.empty(); });
            if (inflight.empty()) {
                if (stop) break;
                continue;
            }
            const int si = inflight.front();
            lk.unlock();
            const int rc = wait_event(slots[si].ev);
            const double t = now_s();
            lk.lock();
            inflight.pop_front();
            Slot& sl = slots[si];
            // a batch that overran its bound may still be running: its
            // requests fail but its pool ranges and slot stay held
            const bool release = rc != BSG_ERR_TIMEOUT;
            for (Request* q : sl.reqs) complete(q, rc, t, release);
            sl.reqs.clear();
            if (release) sl.busy = false;
            free_gen++;
            cv_done.notify_all();
            cv_disp.notify_one();
        }
    }
};

namespace {

void destroy_resources(bsg_server* s) {
    for (auto& sl : s->slots) {
        if (sl.st) cudaStreamSynchronize(sl.st);
        if (sl.ev) cudaEventDestroy(sl.ev);
        if (sl.h_tab) cudaFreeHost(sl.h_tab);
        if (sl.d_tab) cudaFree(sl.d_tab);
        if (sl.d_cursor) cudaFree(sl.d_cursor);
        if (sl.st) cudaStreamDestroy(sl.st);
    }
    s->slots.clear();
    if (s->pst) {
        if (s->ctl_h) __atomic_store_n(&s->ctl_h->stop, 1u, __ATOMIC_RELEASE);
        cudaStreamSynchronize(s->pst);  // blocks see stop at their next idle check
        cudaStreamDestroy(s->pst);
        s->pst = nullptr;
    }
    if (s->pev) cudaEventDestroy(s->pev);
    s->pev = nullptr;
    if (s->ring_h) cudaFreeHost(s->ring_h);
    if (s->ctl_h) cudaFreeHost(s->ctl_h);
    if (s->d_cur) cudaFree(s->d_cur);
    if (s->d_taken) cudaFree(s->d_taken);
    if (s->d_done) cudaFree(s->d_done);
    s->ring_h = nullptr;
    s->ctl_h = nullptr;
    s->d_cur = nullptr;
    s->d_taken = nullptr;
    s->d_done = nullptr;
    for (auto& h : s->hosts)
        if (h.owned) cudaHostUnregister(reinterpret_cast<void*>(h.b));
    s->hosts.clear();
    if (s->d_pool) cudaFree(s->d_pool);
    s->d_pool = nullptr;
}

int submit_impl(bsg_server* s, const bsg_request* r, uint64_t* id, bool auto_release,
                double t_ref, double* lat_slot) {
    if (!s || !r) return BSG_ERR_INVALID_ARG;
    if (r->n && (!r->sptprice || !r->strike || !r->rate || !r->volatility || !r->otime ||
                 !r->otype || !r->prices))
        return BSG_ERR_INVALID_ARG;
    const uint64_t span = (r->n + kAlign - 1) / kAlign * kAlign;
    if (span > s->cap) return BSG_ERR_BUDGET;
    if (s->persistent && r->n > (uint64_t)kMaxRequestTiles * kTile) return BSG_ERR_CAPACITY;
    Request* q = new (std::nothrow) Request();
    if (!q) return BSG_ERR_OUT_OF_MEMORY;
    q->r = *r;
    q->span = span;
    q->t_ref = t_ref;
    q->auto_release = auto_release;
    q->lat_slot = lat_slot;
    std::lock_guard<std::mutex> lk(s->mu);
    if (!s->cfg.plain && r->n) {
        bool vec = true;
        const size_t b = r->n * 4;
        const void* arrs[7] = {r->sptprice, r->strike, r->rate, r->volatility,
                               r->otime, r->otype, r->prices};
        for (int j = 0; j < 7; ++j) {
            const HostRange* h = s->host_range(arrs[j], b);
            if (!h) {
                delete q;
                return BSG_ERR_INVALID_ARG;  // not inside registered host memory
            }
            const uintptr_t dev = reinterpret_cast<uintptr_t>(arrs[j]) + h->delta;
            if ((dev & 15) != 0) vec = false;
            if (j < 5) q->desc.src[j] = reinterpret_cast<const float*>(dev);
            else if (j == 5) q->desc.ot = reinterpret_cast<const int32_t*>(dev);
            else q->desc.out = reinterpret_cast<float*>(dev);
        }
        q->desc.vec = vec ? 1 : 0;
    }
    if (s->stop || s->broken) {
        delete q;
        return BSG_ERR_STATE;
    }
    q->id = s->next_id++;
    s->reqs[q->id] = q;
    s->st.submitted++;
    if (id) *id = q->id;
    if (r->n == 0) {
        s->complete(q, BSG_OK, now_s(), false);
        s->cv_done.notify_all();
        return BSG_OK;
    }
    q->state = Q_QUEUED;
    uint64_t off;
    if (s->persistent && !s->paused && s->queue.empty() && s->can_publish(q, &off)) {
        // nothing ahead of it: publish from this thread (no dispatcher hop);
        // the completer (re)launches the kernel if none is running, so a
        // submitting thread never waits in the CUDA driver
        s->publish(q, off);
        s->cv_comp.notify_one();
        return BSG_OK;
    }
    s->queue.push_back(q);
    s->cv_disp.notify_one();
    return BSG_OK;
}

}  // namespace

extern "C" {

int bsg_server_create(bsg_server** out, const bsg_server_config* cfg) {
    if (!out || !cfg) return BSG_ERR_INVALID_ARG;
    *out = nullptr;
    if (cfg->max_inflight < 1 || cfg->max_inflight > 16 || cfg->max_batch_requests < 0 ||
        cfg->max_batch_requests > 65536 || cfg->budget_bytes < 28 * kAlign ||
        (cfg->persistent_blocks != 0 && (cfg->persistent_blocks < 8 || cfg->persistent_blocks > 4096)) ||
        cfg->persistent_window < 0 || cfg->persistent_window > (int)kMaxWindow)
        return BSG_ERR_INVALID_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || cfg->device < 0 || cfg->device >= ndev) {
        cudaGetLastError();
        return BSG_ERR_NO_DEVICE;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, cfg->device) != cudaSuccess ||
        !(prop.major == 10 && prop.minor == 3))
        return BSG_ERR_NO_DEVICE;
    bsg_server* s = new (std::nothrow) bsg_server();
    if (!s) return BSG_ERR_OUT_OF_MEMORY;
    s->cfg = *cfg;
    s->device = cfg->device;
    s->sm_count = prop.multiProcessorCount;
    s->max_req = cfg->max_batch_requests ? cfg->max_batch_requests : 4096;
    s->batch_timeout = cfg->batch_timeout_s > 0 ? cfg->batch_timeout_s : 30.0;
    switch (cfg->flags & BSG_MODE_MASK) {
        case BSG_MODE_FAST: s->mode = bsg::MODE_FAST; break;
        case BSG_MODE_SFU_REF: s->mode = bsg::MODE_SFU_REF; break;
        case BSG_MODE_LIBM_REF: s->mode = bsg::MODE_LIBM_REF; break;
        default: delete s; return BSG_ERR_INVALID_ARG;
    }
    s->batch_grid = s->sm_count * bsg::batch_blocks_per_sm();
    s->persistent = !cfg->plain && cfg->fused == 2;
    int rc = BSG_OK;
    do {
        if (cudaSetDevice(s->device) != cudaSuccess) { rc = BSG_ERR_NO_DEVICE; break; }
        s->cap = cfg->budget_bytes / 28 / kAlign * kAlign;
        s->free_list[0] = s->cap;
        if (s->persistent) {
            // the GPU reads requests from, and counts tiles into, pinned host
            // memory with system-scope atomics: the host must support them
            int native = 0;
            if (cudaDeviceGetAttribute(&native, cudaDevAttrHostNativeAtomicSupported, s->device) !=
                    cudaSuccess || !native) { rc = BSG_ERR_NOT_SUPPORTED; break; }
            if (cudaHostAlloc(reinterpret_cast<void**>(&s->ring_h), kRing * sizeof(PEntry),
                              cudaHostAllocMapped) != cudaSuccess ||
                cudaHostAlloc(reinterpret_cast<void**>(&s->ctl_h), sizeof(PCtl), cudaHostAllocMapped) !=
                    cudaSuccess ||
                cudaMalloc(&s->d_cur, 2 * sizeof(unsigned long long)) != cudaSuccess ||
                cudaMalloc(&s->d_taken, kRing * sizeof(unsigned long long)) != cudaSuccess ||
                cudaMalloc(&s->d_done, kRing * sizeof(unsigned)) != cudaSuccess) {
                rc = BSG_ERR_OUT_OF_MEMORY;
                break;
            }
            std::memset(s->ring_h, 0, kRing * sizeof(PEntry));
            std::memset(s->ctl_h, 0, sizeof(PCtl));
            // every slot starts armed for the lap before the first: request
            // i (< kRing) finds tag i - kRing and arms the slot for itself
            std::vector<unsigned long long> arm(kRing);
            for (uint64_t i = 0; i < kRing; ++i) arm[i] = bsg_ring::initial_word(i, kRing);
            if (cudaMemcpy(s->d_taken, arm.data(), kRing * sizeof(unsigned long long),
                           cudaMemcpyHostToDevice) != cudaSuccess ||
                cudaMemset(s->d_done, 0, kRing * sizeof(unsigned)) != cudaSuccess) {
                rc = BSG_ERR_CUDA;
                break;
            }
            if (cudaHostGetDevicePointer(reinterpret_cast<void**>(&s->ring_d), s->ring_h, 0) != cudaSuccess ||
                cudaHostGetDevicePointer(reinterpret_cast<void**>(&s->ctl_d), s->ctl_h, 0) != cudaSuccess ||
                cudaMemset(s->d_cur, 0, 2 * sizeof(unsigned long long)) != cudaSuccess ||
                cudaStreamCreateWithFlags(&s->pst, cudaStreamNonBlocking) != cudaSuccess ||
                cudaEventCreateWithFlags(&s->pev, cudaEventDisableTiming) != cudaSuccess ||
                cudaDeviceSynchronize() != cudaSuccess) {
                rc = BSG_ERR_CUDA;
                break;
            }
            int occ = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, serve_persistent_kernel<bsg::MODE_FAST>,
                                                              kThreads, 0) != cudaSuccess || occ < 1)
                occ = 1;
            // enough blocks to keep the host link busy: each block has one
            // 2048-option tile (49 KB) in flight, and a tile takes ~10 us
            // on a loaded link, so the link needs ~40+ blocks; 3 per SM
            s->pgrid = cfg->persistent_blocks ? (unsigned)cfg->persistent_blocks
                                              : (unsigned)(s->sm_count * std::min(occ, 3));
            s->pwindow = cfg->persistent_window ? (unsigned long long)cfg->persistent_window
                                                : kDefaultWindow;
            break;  // no device pool and no batch slots on this path
        }
        // the device pool holds requests only on the unfused and plain paths;
        // the fused kernel reads and writes host memory in place
        if (cfg->plain || cfg->fused == 0) {
            if (cudaMalloc(&s->d_pool, s->cap * 28) != cudaSuccess) { rc = BSG_ERR_OUT_OF_MEMORY; break; }
            float* f = reinterpret_cast<float*>(s->d_pool);
            const uint64_t c = s->cap;
            s->pool = bsg::SoA{f, f + c, f + 2 * c, f + 3 * c, f + 4 * c,
                               reinterpret_cast<const int32_t*>(f + 5 * c), f + 6 * c};
        }
        const int nslots = cfg->plain ? 1 : cfg->max_inflight;
        s->slots.resize(nslots);
        const size_t tb = table_bytes(s->max_req);
        for (auto& sl : s->slots) {
            if (cudaStreamCreateWithFlags(&sl.st, cudaStreamNonBlocking) != cudaSuccess ||
                cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming) != cudaSuccess) {
                rc = BSG_ERR_CUDA;
                break;
            }
            if (cudaMallocHost(&sl.h_tab, tb) != cudaSuccess || cudaMalloc(&sl.d_tab, tb) != cudaSuccess ||
                cudaMalloc(&sl.d_cursor, 256) != cudaSuccess ||
                cudaMemset(sl.d_cursor, 0, 256) != cudaSuccess) {
                rc = BSG_ERR_OUT_OF_MEMORY;
                break;
            }
        }
    } while (0);
    if (rc != BSG_OK) {
        cudaGetLastError();
        destroy_resources(s);
        delete s;
        return rc;
    }
    s->disp = std::thread([s] { s->dispatcher(); });
    s->comp = std::thread([s] { s->completer(); });
    *out = s;
    return BSG_OK;
}

void bsg_server_destroy(bsg_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        const double t = now_s();
        while (!s->queue.empty()) {
            Request* q = s->queue.front();
            s->queue.pop_front();
            s->complete(q, BSG_ERR_CANCELLED, t, false);
        }
    }
    // let in-flight batches complete, then stop the threads
    {
        std::unique_lock<std::mutex> lk(s->mu);
        s->cv_done.wait_for(lk, std::chrono::duration<double>(s->batch_timeout + 1.0),
                            [&] { return s->inflight.empty() && s->pinflight.empty(); });
        s->stop = true;
    }
    s->cv_disp.notify_all();
    s->cv_comp.notify_all();
    if (s->disp.joinable()) s->disp.join();
    if (s->comp.joinable()) s->comp.join();
    cudaSetDevice(s->device);
    destroy_resources(s);
    for (auto& kv : s->reqs) delete kv.second;
    s->reqs.clear();
    delete s;
}

int bsg_server_register(bsg_server* s, void* ptr, size_t bytes) {
    if (!s || !ptr || !bytes) return BSG_ERR_INVALID_ARG;
    cudaSetDevice(s->device);
    bool owned = false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) cudaGetLastError();
    else if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged)
        return BSG_ERR_INVALID_ARG;
    if (!(cudaPointerGetAttributes(&a, ptr) == cudaSuccess && a.type == cudaMemoryTypeHost)) {
        cudaGetLastError();
        const cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterMapped);
        if (e == cudaErrorHostMemoryAlreadyRegistered) {
            cudaGetLastError();
        } else if (e != cudaSuccess) {
            cudaGetLastError();
            return BSG_ERR_CUDA;
        } else {
            owned = true;
        }
    }
    if (!owned) {
        // already pinned by someone else: the whole range must lie inside
        // that allocation, or the GPU could touch unpinned pages
        uintptr_t rb = 0;
        size_t rs = 0;
        const uintptr_t pb = reinterpret_cast<uintptr_t>(ptr);
        if (!cuda_range(ptr, &rb, &rs) || pb < rb || pb + bytes > rb + rs) {
            cudaGetLastError();
            return BSG_ERR_INVALID_ARG;
        }
    }
    void* dptr = nullptr;
    if (cudaHostGetDevicePointer(&dptr, ptr, 0) != cudaSuccess || !dptr) {
        cudaGetLastError();
        if (owned) cudaHostUnregister(ptr);
        return BSG_ERR_CUDA;
    }
    HostRange h;
    h.b = reinterpret_cast<uintptr_t>(ptr);
    h.e = h.b + bytes;
    h.delta = reinterpret_cast<intptr_t>(dptr) - static_cast<intptr_t>(h.b);
    h.owned = owned;
    std::lock_guard<std::mutex> lk(s->mu);
    s->hosts.push_back(h);
    return BSG_OK;
}

int bsg_server_submit(bsg_server* s, const bsg_request* r, uint64_t* id) {
    return submit_impl(s, r, id, false, now_s(), nullptr);
}

int bsg_server_wait(bsg_server* s, uint64_t id, double timeout_s, double* latency_s) {
    if (!s) return BSG_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return BSG_ERR_INVALID_ARG;
    Request* q = it->second;
    auto done = [&] { return q->state == Q_DONE; };
    if (timeout_s < 0) s->cv_done.wait(lk, done);
    else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done))
        return BSG_ERR_TIMEOUT;
    const int status = q->status;
    if (latency_s) *latency_s = q->t_done - q->t_ref;
    s->reqs.erase(id);
    delete q;
    return status;
}

int bsg_server_cancel(bsg_server* s, uint64_t id) {
    if (!s) return BSG_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return BSG_ERR_INVALID_ARG;
    Request* q = it->second;
    if (q->state != Q_QUEUED) return BSG_ERR_STATE;
    s->queue.erase(std::find(s->queue.begin(), s->queue.end(), q));
    s->complete(q, BSG_ERR_CANCELLED, now_s(), false);
    s->cv_done.notify_all();
    s->cv_disp.notify_one();
    return BSG_OK;
}

int bsg_server_pause(bsg_server* s, int paused) {
    if (!s) return BSG_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    s->paused = paused != 0;
    s->cv_disp.notify_one();
    return BSG_OK;
}

int bsg_server_get_stats(bsg_server* s, bsg_server_stats* out) {
    if (!s || !out) return BSG_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->st;
    out->queued = s->queue.size();
    uint64_t in = s->pinflight.size();  // persistent path: published, not complete
    for (int si : s->inflight) in += s->slots[si].reqs.size();
    out->inflight_requests = in;
    return BSG_OK;
}

int bsg_serve_trace(const bsg_server_config* cfg, const bsg_trace_config* tr,
                    bsg_trace_result* out, double* lat_out, size_t lat_cap) {
    if (!cfg || !tr || !out) return BSG_ERR_INVALID_ARG;
    if (!(tr->rate_per_s > 0) || !(tr->duration_s > 0) || tr->min_n < 1 || tr->max_n < tr->min_n ||
        tr->max_n > tr->pool_n || !tr->sptprice || !tr->strike || !tr->rate || !tr->volatility ||
        !tr->otime || !tr->otype || !tr->prices)
        return BSG_ERR_INVALID_ARG;
    std::memset(out, 0, sizeof(*out));
    // the arrival schedule (Poisson), sizes (log-uniform) and pool offsets
    std::mt19937_64 rng(tr->seed);
    std::exponential_distribution<double> gap(tr->rate_per_s);
    std::uniform_real_distribution<double> u(0.0, 1.0);
    std::vector<double> at;
    std::vector<uint64_t> ns, offs;
    const double lmin = std::log((double)tr->min_n), lmax = std::log((double)tr->max_n + 1.0);
    for (double t = gap(rng); t < tr->duration_s; t += gap(rng)) {
        uint64_t n = (uint64_t)std::floor(std::exp(lmin + (lmax - lmin) * u(rng)));
        n = std::min<uint64_t>(std::max<uint64_t>(n, tr->min_n), tr->max_n);
        const uint64_t room = tr->pool_n - n;
        const uint64_t o = (uint64_t)(u(rng) * (double)(room + 1)) & ~3ull;
        at.push_back(t);
        ns.push_back(n);
        offs.push_back(std::min(o, room));
    }
    const size_t count = at.size();
    std::vector<double> lat(count, NAN);
    bsg_server* s = nullptr;
    int rc = bsg_server_create(&s, cfg);
    if (rc) return rc;
    const size_t pb = tr->pool_n * 4;
    const void* arrs[7] = {tr->sptprice, tr->strike, tr->rate, tr->volatility, tr->otime,
                           tr->otype, tr->prices};
    for (int j = 0; j < 7 && rc == BSG_OK; ++j) rc = bsg_server_register(s, const_cast<void*>(arrs[j]), pb);
    if (rc) {
        bsg_server_destroy(s);
        return rc;
    }
    const double t0 = now_s() + 0.02;
    double late = 0.0;
    size_t late_at = 0;
    uint64_t submitted = 0;
    for (size_t k = 0; k < count; ++k) {
        const double ts = t0 + at[k];
        double tn = now_s();
        if (tn < ts) {
            if (ts - tn > 200e-6)
                std::this_thread::sleep_for(std::chrono::duration<double>(ts - tn - 100e-6));
            while (now_s() < ts) {
            }
        } else if (tn - ts > late) {
            late = tn - ts;
            late_at = k;
        }
        const uint64_t o = offs[k];
        bsg_request r{tr->sptprice + o, tr->strike + o, tr->rate + o, tr->volatility + o,
                      tr->otime + o, tr->otype + o, tr->prices + o, ns[k]};
        if (submit_impl(s, &r, nullptr, true, ts, &lat[k]) == BSG_OK) submitted++;
    }
    // drain (bounded)
    const double drain = tr->drain_timeout_s > 0 ? tr->drain_timeout_s : 60.0;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        s->cv_done.wait_for(lk, std::chrono::duration<double>(drain), [&] {
            return s->st.completed + s->st.failed + s->st.cancelled >= submitted;
        });
    }
    if (const char* dbg = std::getenv("BSG_TRACE_DEBUG"); dbg && *dbg == '1')
        std::fprintf(stderr, "bsg_serve_trace: submitter at most %.3f ms late, at request %zu of %zu "
                             "(scheduled %.3f s into the trace)\n",
                     late * 1e3, late_at, count, count ? at[late_at] : 0.0);
    bsg_server_stats stt;
    bsg_server_get_stats(s, &stt);
    bsg_server_destroy(s);  // cancels anything left
    // statistics over completed requests
    std::vector<double> ok;
    ok.reserve(count);
    uint64_t opts = 0;
    double t_last = t0;
    for (size_t k = 0; k < count; ++k) {
        if (std::isnan(lat[k])) continue;
        ok.push_back(lat[k]);
        opts += ns[k];
        t_last = std::max(t_last, t0 + at[k] + lat[k]);
    }
    std::sort(ok.begin(), ok.end());
    auto pct = [&](double p) -> double {
        if (ok.empty()) return (double)NAN;
        size_t i = (size_t)std::ceil(p * (double)ok.size()) - 1;
        return ok[std::min(i, ok.size() - 1)];
    };
    out->requests = count;
    out->completed = ok.size();
    out->failed = count - ok.size();
    out->options = opts;
    out->wall_s = t_last - t0;
    out->options_per_s = out->wall_s > 0 ? (double)opts / out->wall_s : 0.0;
    out->requests_per_s = out->wall_s > 0 ? (double)ok.size() / out->wall_s : 0.0;
    out->p50_s = pct(0.50);
    out->p99_s = pct(0.99);
    out->p999_s = pct(0.999);
    out->max_s = ok.empty() ? NAN : ok.back();
    double sum = 0;
    for (double x : ok) sum += x;
    out->mean_s = ok.empty() ? NAN : sum / (double)ok.size();
    out->batches = stt.batches;
    out->mean_batch_requests = stt.batches ? (double)stt.completed / (double)stt.batches : 0.0;
    out->late_submit_max_s = late;
    if (lat_out)
        for (size_t k = 0; k < std::min(lat_cap, count); ++k) lat_out[k] = lat[k];
    return BSG_OK;
}

}  // extern "C"
