// bsg_kernels.cu -- sm_103a kernels of the Black-Scholes map.
//
// The hot path is an HBM-bound elementwise map: 28 bytes per option per run
// (five float inputs, one int32 otype, one float price) against ~86 issued
// instructions (the FAST arithmetic runs two options per packed f32x2
// instruction).  Design:
//  * SoA streams read with 128-bit (v4) or 256-bit (v8) non-coherent loads
//    that do not allocate in L1, optionally inserted into L2 as evict_first
//    (a cyclic scan of a working set larger than L2 then keeps a slice of it
//    resident between passes), or with a prefix of the book (a tuned
//    fraction of the L2, inputs and prices) evict_last and the rest evict_first, so that
//    the prefix stays resident from pass to pass; prices stored with
//    streaming stores (or with the prefix's policy).
//  * Each thread loads VPT vector groups of all six arrays before computing,
//    so a warp keeps 6 * VPT independent 512/1024-byte requests in flight.
//  * Grid: one block per tile, or a persistent grid-stride loop sized in
//    multiples of the SM count (chosen by the autotuner).
//  * No shared memory, no tensor cores: there is no reuse to stage and no
//    contraction to run.
#include "bsg_internal.h"
#include "bsg_math.cuh"

#include <atomic>

namespace bsg {

// ------------------------------------------------------------ memory access
__device__ __forceinline__ unsigned long long evict_first_policy() {
    unsigned long long pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ unsigned long long evict_last_policy() {
    unsigned long long pol;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

template <int W>
struct Raw {
    uint32_t v[W];
};

// Load paths of the vector kernel: LP 0/2: ld.global.nc.L1::no_allocate
// (v4 / v8); LP 1 / 6: the same v4 / v8 loads with an L2 evict_first cache
// policy; LP 7: v8 loads and stores of a resident prefix of the book (the
// first `gres` groups, a tuned fraction of the L2) with an evict_last
// policy, the rest evict_first -- the prefix then stays in L2 from pass to
// pass while the rest streams through.
// LP 8: the v8 loads of LP 2 and stores with the default L2 policy, every
// other pass in reverse tile order (the L2 keeps what it saw last).
__host__ __device__ constexpr bool lp_resident(int lp) { return lp == 7; }
__host__ __device__ constexpr bool lp_hinted(int lp) { return lp == 1 || lp == 6 || lp == 7; }
__host__ __device__ constexpr bool lp_evict_first(int lp) { return lp == 1 || lp == 6; }
__host__ __device__ constexpr bool lp_v8(int lp) { return lp == 2 || lp == 6 || lp == 7 || lp == 8; }
__host__ __device__ constexpr bool lp_alternating(int lp) { return lp == 8; }

template <int W, int LP>
__device__ __forceinline__ Raw<W> ld_group(const void* p, unsigned long long pol) {
    Raw<W> r;
    if constexpr (W == 4) {
        if constexpr (LP == 1) {
            asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.u32 {%0,%1,%2,%3}, [%4], %5;"
                : "=r"(r.v[0]), "=r"(r.v[1]), "=r"(r.v[2]), "=r"(r.v[3])
                : "l"(p), "l"(pol));
        } else {
            (void)pol;
            asm("ld.global.nc.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
                : "=r"(r.v[0]), "=r"(r.v[1]), "=r"(r.v[2]), "=r"(r.v[3])
                : "l"(p));
        }
    } else if constexpr (lp_hinted(LP)) {
        asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8], %9;"
            : "=r"(r.v[0]), "=r"(r.v[1]), "=r"(r.v[2]), "=r"(r.v[3]),
              "=r"(r.v[4]), "=r"(r.v[5]), "=r"(r.v[6]), "=r"(r.v[7])
            : "l"(p), "l"(pol));
    } else {
        (void)pol;
        asm("ld.global.nc.L1::no_allocate.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
            : "=r"(r.v[0]), "=r"(r.v[1]), "=r"(r.v[2]), "=r"(r.v[3]),
              "=r"(r.v[4]), "=r"(r.v[5]), "=r"(r.v[6]), "=r"(r.v[7])
            : "l"(p));
    }
    return r;
}

template <int W, int LP>
__device__ __forceinline__ void st_group(float* p, const float (&x)[W], unsigned long long pol) {
    if constexpr (W == 8 && lp_resident(LP)) {
        asm volatile("st.global.L2::cache_hint.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8}, %9;"
                     :: "l"(p), "f"(x[0]), "f"(x[1]), "f"(x[2]), "f"(x[3]),
                        "f"(x[4]), "f"(x[5]), "f"(x[6]), "f"(x[7]), "l"(pol)
                     : "memory");
    } else if constexpr (W == 8 && lp_alternating(LP)) {
        (void)pol;
        asm volatile("st.global.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};"
                     :: "l"(p), "f"(x[0]), "f"(x[1]), "f"(x[2]), "f"(x[3]),
                        "f"(x[4]), "f"(x[5]), "f"(x[6]), "f"(x[7])
                     : "memory");
    } else if constexpr (W == 4) {
        (void)pol;
        asm volatile("st.global.cs.v4.f32 [%0], {%1,%2,%3,%4};"
                     :: "l"(p), "f"(x[0]), "f"(x[1]), "f"(x[2]), "f"(x[3])
                     : "memory");
    } else {
        asm volatile("st.global.cs.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};"
                     :: "l"(p), "f"(x[0]), "f"(x[1]), "f"(x[2]), "f"(x[3]),
                        "f"(x[4]), "f"(x[5]), "f"(x[6]), "f"(x[7])
                     : "memory");
    }
}


template <int M>
__device__ __forceinline__ void price_scalar(const SoA& a, int64_t i) {
    a.out[i] = price<M>(__ldg(a.s + i), __ldg(a.k + i), __ldg(a.r + i),
                        __ldg(a.v + i), __ldg(a.t + i), __ldg(a.ot + i));
}

// Prices vector groups [g0, g1) (group = W options) of one block's range:
// each thread loads VPT groups (stride blockDim.x) of all six arrays, then
// computes and stores them.  pol is the L2 policy of the hinted load paths;
// for LP 7, groups below gres use pol_res instead.
template <int M, int W, int VPT, int LP>
__device__ __forceinline__ void price_groups(const SoA& a, int64_t g0, int64_t g1,
                                             unsigned long long pol,
                                             unsigned long long pol_res, int64_t gres) {
    const int64_t bd = blockDim.x;
    for (int64_t base = g0; base < g1; base += bd * VPT) {
        Raw<W> S[VPT], K[VPT], R[VPT], V[VPT], T[VPT], O[VPT];
#pragma unroll
        for (int j = 0; j < VPT; ++j) {
            const int64_t g = base + threadIdx.x + j * bd;
            if (g < g1) {
                const int64_t o = g * W;
                const unsigned long long pl = (lp_resident(LP) && g < gres) ? pol_res : pol;
                S[j] = ld_group<W, LP>(a.s + o, pl);
                K[j] = ld_group<W, LP>(a.k + o, pl);
                R[j] = ld_group<W, LP>(a.r + o, pl);
                V[j] = ld_group<W, LP>(a.v + o, pl);
                T[j] = ld_group<W, LP>(a.t + o, pl);
                O[j] = ld_group<W, LP>(a.ot + o, pl);
            }
        }
#pragma unroll
        for (int j = 0; j < VPT; ++j) {
            const int64_t g = base + threadIdx.x + j * bd;
            if (g < g1) {
                float p[W];
#pragma unroll
                for (int e = 0; e < W; e += 4) {
                    const float4 q = price4<M>(
                        make_float4(__uint_as_float(S[j].v[e]), __uint_as_float(S[j].v[e + 1]),
                                    __uint_as_float(S[j].v[e + 2]), __uint_as_float(S[j].v[e + 3])),
                        make_float4(__uint_as_float(K[j].v[e]), __uint_as_float(K[j].v[e + 1]),
                                    __uint_as_float(K[j].v[e + 2]), __uint_as_float(K[j].v[e + 3])),
                        make_float4(__uint_as_float(R[j].v[e]), __uint_as_float(R[j].v[e + 1]),
                                    __uint_as_float(R[j].v[e + 2]), __uint_as_float(R[j].v[e + 3])),
                        make_float4(__uint_as_float(V[j].v[e]), __uint_as_float(V[j].v[e + 1]),
                                    __uint_as_float(V[j].v[e + 2]), __uint_as_float(V[j].v[e + 3])),
                        make_float4(__uint_as_float(T[j].v[e]), __uint_as_float(T[j].v[e + 1]),
                                    __uint_as_float(T[j].v[e + 2]), __uint_as_float(T[j].v[e + 3])),
                        make_int4((int)O[j].v[e], (int)O[j].v[e + 1], (int)O[j].v[e + 2],
                                  (int)O[j].v[e + 3]));
                    p[e] = q.x;
                    p[e + 1] = q.y;
                    p[e + 2] = q.z;
                    p[e + 3] = q.w;
                }
                const unsigned long long pst = (lp_resident(LP) && g < gres) ? pol_res : pol;
                st_group<W, LP>(a.out + g * W, p, pst);
            }
        }
    }
}

// ------------------------------------------------------------- plain map
// Vector kernel: options [0, n - n % W) in groups of W; the last n % W
// options by block 0.  blocks_per_sm == 0: each block prices one tile of
// blockDim.x * VPT groups; otherwise blocks stride over tiles.
// Programmatic dependent launch: every block lets the next pass launch as
// soon as it starts (the next pass reads only the inputs, which no pass
// writes), and waits for the previous pass to complete only after its own
// stores, so a pass still completes after the one before it.  Both
// instructions are no-ops for a launch without the PDL attribute.
// Registers: one-group shapes (VPT = 1) are held to 64 per thread (1024
// threads per SM, no spills); more groups per thread need up to 128.  The
// reference-order libm mode (compute-bound, float-float exp/log) always runs
// 256-thread blocks, four per SM (59 registers, no spills).
__device__ __forceinline__ void pdl_trigger() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_wait() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

template <int M, int W, int VPT, int LP>
__global__ void __launch_bounds__(M == MODE_LIBM_REF ? 256 : 512,
                                  M == MODE_LIBM_REF ? 4 : (VPT == 1 ? 2 : 1))
    map_vec_kernel(SoA a, int64_t n, int64_t gres, int rev) {
    pdl_trigger();
    const unsigned long long pol =
        (lp_evict_first(LP) || lp_resident(LP)) ? evict_first_policy() : 0ull;
    const unsigned long long pol_res = lp_resident(LP) ? evict_last_policy() : 0ull;
    const int64_t ngroups = n / W;
    const int64_t tile = (int64_t)blockDim.x * VPT;
    const int64_t ntiles = (ngroups + tile - 1) / tile;
    for (int64_t ti = blockIdx.x; ti < ntiles; ti += gridDim.x) {
        // LP 8's odd passes take the tiles from the last to the first
        const int64_t t0 = (lp_alternating(LP) && rev ? ntiles - 1 - ti : ti) * tile;
        const int64_t t1 = (t0 + tile < ngroups) ? t0 + tile : ngroups;
        price_groups<M, W, VPT, LP>(a, t0, t1, pol, pol_res, gres);
    }
    if (blockIdx.x == 0) {
        const int64_t i = ngroups * W + threadIdx.x;
        if (i < n) price_scalar<M>(a, i);
    }
    pdl_wait();
}

// Scalar kernel: any 4-byte aligned pointers.
template <int M>
__global__ void __launch_bounds__(256) map_scalar_kernel(SoA a, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        price_scalar<M>(a, i);
}

// ------------------------------------------------- TMA bulk-staged variant
// Each persistent CTA streams whole tiles (256 threads x OPT options) through
// a STAGES-deep ring in shared memory: one thread issues six 1D bulk copies
// (cp.async.bulk, one per input array) per tile, completing on the stage's
// mbarrier with a transaction count; every thread waits on the barrier,
// prices OPT options from shared memory and stores them with streaming
// stores.  A stage is refilled after a block barrier and a proxy fence.
// Waits are bounded: on expiry the CTA records kErrBulkTimeout in
// g_bulk_err, waits (bounded) for its copies in flight and returns.
// Shapes: <8, 3> 144 KB per CTA (1 per SM), <4, 4> 96 KB (2 per SM),
// <4, 3> 72 KB (3 per SM).
constexpr int kBulkThreads = 256;
constexpr unsigned kErrBulkTimeout = 1u;
constexpr uint64_t kBulkWaitNs = 1000000000ull;  // bound of one wait: 1 s

// Error word of the bulk kernels (kErrBulkTimeout); read and cleared by the
// host with bulk_error_take().
__device__ unsigned g_bulk_err;

template <int OPT, int STAGES>
struct BulkShape {
    static constexpr int tile = kBulkThreads * OPT;
    static constexpr int stage_bytes = 6 * tile * 4;
    static constexpr int smem = STAGES * stage_bytes;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok) : "r"(bar), "r"(parity) : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits for the phase of `bar` with parity `parity` for at most limit_ns of
// wall time (the GPU's global timer); false when the bound expired.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, uint64_t limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
}

// One 1D bulk copy of `bytes` (16-byte aligned at both ends, a multiple of
// 16) into shared memory, completing on `bar`, with L2 cache policy `pol`
// (evict_first: the cyclic scan then keeps a slice of the inputs in L2 from
// pass to pass, as the evict_first load paths do).
__device__ __forceinline__ void bulk_copy(char* dst, const char* src, int bytes, uint32_t bar,
                                          unsigned long long pol) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint"
        " [%0], [%1], %2, [%3], %4;"
        :: "r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(bar), "l"(pol) : "memory");
}

// Issues the six copies of tile `tile` into stage memory `st` (thread 0).
// tx_extra (0 in production) raises the barrier's expected byte count above
// what the copies deliver, so that its phase can never complete: the
// self-test of the bounded waits.
template <int TILE>
__device__ __forceinline__ void bulk_issue(const SoA& a, int64_t tile, char* st, uint32_t bar,
                                           uint32_t tx_extra) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                 :: "r"(bar), "r"(6 * TILE * 4 + tx_extra) : "memory");
    const size_t off = (size_t)tile * TILE * 4;
    const unsigned long long pol = evict_first_policy();
    bulk_copy(st + 0 * TILE * 4, reinterpret_cast<const char*>(a.s) + off, TILE * 4, bar, pol);
    bulk_copy(st + 1 * TILE * 4, reinterpret_cast<const char*>(a.k) + off, TILE * 4, bar, pol);
    bulk_copy(st + 2 * TILE * 4, reinterpret_cast<const char*>(a.r) + off, TILE * 4, bar, pol);
    bulk_copy(st + 3 * TILE * 4, reinterpret_cast<const char*>(a.v) + off, TILE * 4, bar, pol);
    bulk_copy(st + 4 * TILE * 4, reinterpret_cast<const char*>(a.t) + off, TILE * 4, bar, pol);
    bulk_copy(st + 5 * TILE * 4, reinterpret_cast<const char*>(a.ot) + off, TILE * 4, bar, pol);
}

template <int M, int OPT, int STAGES>
__global__ void __launch_bounds__(kBulkThreads) map_bulk_kernel(SoA a, int64_t n, uint64_t wait_ns,
                                                                 uint32_t tx_extra) {
    using B = BulkShape<OPT, STAGES>;
    constexpr int TILE = B::tile;
    extern __shared__ __align__(128) char smem[];
    __shared__ __align__(8) unsigned long long bars[STAGES];
    __shared__ int sh_abort;
    pdl_trigger();
    const int64_t ntiles = n / TILE;
    // tiles of this CTA: blockIdx.x + k * gridDim.x
    const int64_t mine = (ntiles > blockIdx.x) ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&bars[s])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        sh_abort = 0;
        for (int s = 0; s < STAGES && s < mine; ++s)
            bulk_issue<TILE>(a, blockIdx.x + (int64_t)s * gridDim.x, smem + s * B::stage_bytes,
                             smem_u32(&bars[s]), tx_extra);
    }
    __syncthreads();
    int64_t k = 0;
    for (; k < mine; ++k) {
        const int s = (int)(k % STAGES);
        const uint32_t parity = (uint32_t)((k / STAGES) & 1);
        const bool ok = mbar_wait_bounded(smem_u32(&bars[s]), parity, wait_ns);
        if (!ok) sh_abort = 1;  // benign race: every writer stores 1
        __syncthreads();
        if (sh_abort) break;
        const char* st = smem + s * B::stage_bytes;
        const int64_t tile = blockIdx.x + k * gridDim.x;
        // thread t prices options 4t..4t+3 of each 1024-option slice, so each
        // 128-bit shared load and global store of a warp covers 512
        // contiguous bytes (no bank conflicts)
        float p[OPT / 4][4];
#pragma unroll
        for (int h = 0; h < OPT / 4; ++h) {
            const int o = (4 * threadIdx.x + 1024 * h) * 4;
            const float4 S = *reinterpret_cast<const float4*>(st + 0 * TILE * 4 + o);
            const float4 K = *reinterpret_cast<const float4*>(st + 1 * TILE * 4 + o);
            const float4 R = *reinterpret_cast<const float4*>(st + 2 * TILE * 4 + o);
            const float4 V = *reinterpret_cast<const float4*>(st + 3 * TILE * 4 + o);
            const float4 T = *reinterpret_cast<const float4*>(st + 4 * TILE * 4 + o);
            const int4 O = *reinterpret_cast<const int4*>(st + 5 * TILE * 4 + o);
            const float4 q = price4<M>(S, K, R, V, T, O);
            p[h][0] = q.x;
            p[h][1] = q.y;
            p[h][2] = q.z;
            p[h][3] = q.w;
        }
        __syncthreads();  // every thread has read stage s
        if (threadIdx.x == 0 && k + STAGES < mine) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            bulk_issue<TILE>(a, blockIdx.x + (k + STAGES) * gridDim.x, smem + s * B::stage_bytes,
                             smem_u32(&bars[s]), tx_extra);
        }
#pragma unroll
        for (int h = 0; h < OPT / 4; ++h)
            st_group<4, 0>(a.out + tile * TILE + 1024 * h + 4 * threadIdx.x, p[h], 0ull);
    }
    if (k < mine) {
        // timed out: record it, let this CTA's copies in flight land (bounded)
        if (threadIdx.x == 0) {
            atomicOr(&g_bulk_err, kErrBulkTimeout);
            for (int64_t q = k; q < mine && q < k + STAGES; ++q)
                mbar_wait_bounded(smem_u32(&bars[q % STAGES]), (uint32_t)((q / STAGES) & 1), wait_ns);
        }
        __syncthreads();
        return;
    }
    // options past the last whole tile: the last CTA, one per thread
    if (blockIdx.x == gridDim.x - 1)
        for (int64_t i = ntiles * TILE + threadIdx.x; i < n; i += kBulkThreads)
            price_scalar<M>(a, i);
    pdl_wait();
}

unsigned bulk_error_take() {
    unsigned v = 0, zero = 0;
    if (cudaMemcpyFromSymbol(&v, g_bulk_err, sizeof v) != cudaSuccess ||
        cudaMemcpyToSymbol(g_bulk_err, &zero, sizeof zero) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return v;
}

static bool aligned(const void* p, uintptr_t al) {
    return (reinterpret_cast<uintptr_t>(p) & (al - 1)) == 0;
}

bool map_vectorizable(const SoA& a, const MapCfg& cfg) {
    // 256-bit loads for LP 2 and 6, and for the bulk paths' small-n fallback
    const uintptr_t al = (cfg.load_path >= 2) ? 32 : 16;
    return aligned(a.s, al) && aligned(a.k, al) && aligned(a.r, al) &&
           aligned(a.v, al) && aligned(a.t, al) && aligned(a.ot, al) &&
           aligned(a.out, al);
}

template <int M, int OPT, int STAGES>
static cudaError_t launch_map_bulk(const SoA& a, int64_t n, const MapCfg& cfg, int sm_count,
                                  cudaStream_t st, uint64_t wait_ns = kBulkWaitNs,
                                  uint32_t tx_extra = 0) {
    using B = BulkShape<OPT, STAGES>;
    // opt in to the dynamic shared memory, once per device (contexts on
    // several host threads may race here: setting the attribute twice is
    // harmless, the bit mask is atomic)
    static std::atomic<unsigned long long> opted{0};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev >= 64 || !(opted.load(std::memory_order_acquire) & (1ull << dev))) {
        e = cudaFuncSetAttribute(map_bulk_kernel<M, OPT, STAGES>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, B::smem);
        if (e != cudaSuccess) return e;
        if (dev < 64) opted.fetch_or(1ull << dev, std::memory_order_release);
    }
    const int64_t ntiles = n / B::tile;
    int64_t grid = (int64_t)sm_count * (220 * 1024 / B::smem);  // CTAs that fit per SM
    if (grid > ntiles) grid = ntiles;
    if (grid < 1) grid = 1;
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)grid);
    lc.blockDim = dim3(kBulkThreads);
    lc.dynamicSmemBytes = B::smem;
    lc.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    lc.attrs = attr;
    lc.numAttrs = cfg.pdl ? 1 : 0;
    return cudaLaunchKernelEx(&lc, map_bulk_kernel<M, OPT, STAGES>, a, n, wait_ns, tx_extra);
}

// The current device's L2 size in bytes (0 if unknown), cached per device.
static int64_t device_l2_bytes() {
    static std::atomic<int64_t> cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
    int64_t v = cache[dev].load(std::memory_order_relaxed);
    if (v == 0) {
        int b = 0;
        if (cudaDeviceGetAttribute(&b, cudaDevAttrL2CacheSize, dev) != cudaSuccess) return 0;
        v = b;
        cache[dev].store(v, std::memory_order_relaxed);
    }
    return v;
}

template <int M>
static cudaError_t launch_map_mode(const SoA& a, int64_t n, const MapCfg& cfg_in,
                                   int sm_count, cudaStream_t st) {
    MapCfg cfg = cfg_in;
    if constexpr (M == MODE_LIBM_REF) {
        // compute-bound (float-float exp/log): 128-bit loads and one
        // 256-thread block per tile (four resident per SM), whatever shape
        // the memory-bound tuning chose
        cfg.load_path = 0;
        cfg.vpt = 1;
        cfg.blocks_per_sm = 0;
        if (cfg.block > 256) cfg.block = 256;
    }
    const int block = cfg.block;
    if (!map_vectorizable(a, cfg)) {
        int64_t grid = (n + 255) / 256;
        const int64_t cap = (int64_t)sm_count * 8;
        if (grid > cap) grid = cap;
        if (grid < 1) grid = 1;
        map_scalar_kernel<M><<<(unsigned)grid, 256, 0, st>>>(a, n);
        return cudaGetLastError();
    }
    if (cfg.load_path >= 3 && cfg.load_path <= 5) {
        if constexpr (M == MODE_FAST) {
            // 3: <8 options, 3 stages>, 4: <4, 4>, 5: <4, 3>
            if (cfg.load_path == 3 && n >= BulkShape<8, 3>::tile)
                return launch_map_bulk<M, 8, 3>(a, n, cfg, sm_count, st);
            if (cfg.load_path == 4 && n >= BulkShape<4, 4>::tile)
                return launch_map_bulk<M, 4, 4>(a, n, cfg, sm_count, st);
            if (cfg.load_path == 5 && n >= BulkShape<4, 3>::tile)
                return launch_map_bulk<M, 4, 3>(a, n, cfg, sm_count, st);
        }
        MapCfg v8 = cfg;  // too small for a whole tile (or another mode): 256-bit loads
        v8.load_path = 2;
        v8.vpt = 1;
        return launch_map_mode<M>(a, n, v8, sm_count, st);
    }
    const int W = lp_v8(cfg.load_path) ? 8 : 4;
    const int64_t ngroups = n / W;
    // LP 7: the first gres groups (res32 32nds of the L2 in inputs and
    // prices, 28 bytes an option) are kept resident across passes
    int64_t gres = 0;
    if (lp_resident(cfg.load_path)) {
        const int res32 = (cfg.res32 >= 1 && cfg.res32 <= 24) ? cfg.res32 : 15;
        gres = device_l2_bytes() * res32 / 32 / (28 * W);
        if (gres > ngroups) gres = ngroups;
    }
    const int64_t tile = (int64_t)block * cfg.vpt;
    int64_t ntiles = (ngroups + tile - 1) / tile;
    int64_t grid = ntiles;
    if (cfg.blocks_per_sm > 0) {
        const int64_t cap = (int64_t)cfg.blocks_per_sm * sm_count;
        if (grid > cap) grid = cap;
    }
    if (grid > 0x7fffffff) grid = 0x7fffffff;
    if (grid < 1) grid = 1;
    const dim3 g((unsigned)grid), b((unsigned)block);

    cudaLaunchConfig_t lc = {};
    lc.gridDim = g;
    lc.blockDim = b;
    lc.dynamicSmemBytes = 0;
    lc.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    lc.attrs = attr;
    lc.numAttrs = cfg.pdl ? 1 : 0;
    cudaError_t le = cudaSuccess;
#define BSG_LAUNCH(W_, V_, L_) \
    le = cudaLaunchKernelEx(&lc, map_vec_kernel<M, W_, V_, L_>, a, n, gres, cfg.rev)
    if constexpr (M == MODE_FAST) {
        switch (cfg.load_path * 10 + cfg.vpt) {
            case 1: BSG_LAUNCH(4, 1, 0); break;
            case 2: BSG_LAUNCH(4, 2, 0); break;
            case 4: BSG_LAUNCH(4, 4, 0); break;
            case 11: BSG_LAUNCH(4, 1, 1); break;
            case 12: BSG_LAUNCH(4, 2, 1); break;
            case 14: BSG_LAUNCH(4, 4, 1); break;
            case 21: BSG_LAUNCH(8, 1, 2); break;
            case 22: BSG_LAUNCH(8, 2, 2); break;
            case 61: BSG_LAUNCH(8, 1, 6); break;
            case 62: BSG_LAUNCH(8, 2, 6); break;
            case 71: BSG_LAUNCH(8, 1, 7); break;
            case 72: BSG_LAUNCH(8, 2, 7); break;
            case 81: BSG_LAUNCH(8, 1, 8); break;
            case 82: BSG_LAUNCH(8, 2, 8); break;
            default: return cudaErrorInvalidValue;
        }
    } else {
        // reference-order paths are validation variants: one shape each.
        if constexpr (M == MODE_LIBM_REF) BSG_LAUNCH(4, 1, 0);
        else if (lp_v8(cfg.load_path)) BSG_LAUNCH(8, 1, 2);
        else BSG_LAUNCH(4, 1, 0);
    }
#undef BSG_LAUNCH
    if (le != cudaSuccess) return le;
    return cudaGetLastError();
}

cudaError_t launch_bulk_wait_selftest(const SoA& a, int64_t n, int sm_count, uint64_t wait_ns,
                                      cudaStream_t st) {
    if (n < BulkShape<4, 4>::tile) return cudaErrorInvalidValue;
    const MapCfg cfg{1, kBulkThreads, 0, 4, 0};
    return launch_map_bulk<MODE_FAST, 4, 4>(a, n, cfg, sm_count, st, wait_ns, 16u);
}

cudaError_t launch_map(const SoA& a, int64_t n, int mode, const MapCfg& cfg,
                       int sm_count, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (cfg.block < 32 || cfg.block > 512 || (cfg.block & 31)) return cudaErrorInvalidValue;
    switch (mode) {
        case MODE_FAST: return launch_map_mode<MODE_FAST>(a, n, cfg, sm_count, st);
        case MODE_SFU_REF: return launch_map_mode<MODE_SFU_REF>(a, n, cfg, sm_count, st);
        case MODE_LIBM_REF: return launch_map_mode<MODE_LIBM_REF>(a, n, cfg, sm_count, st);
        default: return cudaErrorInvalidValue;
    }
}

// ------------------------------------------------------------------ FP64
__global__ void __launch_bounds__(256) fp64_kernel(SoA a, double* out, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = price_fp64(a.s[i], a.k[i], a.r[i], a.v[i], a.t[i], a.ot[i]);
}

// FP64 product mode: double storage in and out (the SIMD variant's NCO = 2
// types), 52 bytes per option; bound by GB300's FP64 rate, not by HBM.
__global__ void __launch_bounds__(256) map_f64_kernel(SoA64 a, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        a.out[i] = price_fp64(__ldg(a.s + i), __ldg(a.k + i), __ldg(a.r + i), __ldg(a.v + i),
                              __ldg(a.t + i), __ldg(a.ot + i));
}

cudaError_t launch_map_f64(const SoA64& a, int64_t n, int sm_count, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    int64_t grid = (n + 255) / 256;
    const int64_t cap = (int64_t)sm_count * 8;
    if (grid > cap) grid = cap;
    map_f64_kernel<<<(unsigned)grid, 256, 0, st>>>(a, n);
    return cudaGetLastError();
}

cudaError_t launch_fp64(const SoA& a, double* out, int64_t n, int sm_count,
                        cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    int64_t grid = (n + 255) / 256;
    const int64_t cap = (int64_t)sm_count * 8;
    if (grid > cap) grid = cap;
    fp64_kernel<<<(unsigned)grid, 256, 0, st>>>(a, out, n);
    return cudaGetLastError();
}

// ------------------------------------------------------------ batched books
// A tile is 8192 options; a block covers it in passes of kBatchBlock
// threads x kBatchVpt v4 groups.
constexpr int kBatchVpt = 1;
constexpr uint64_t kBatchTileOptions = 8192;

uint64_t batch_tile_options() { return kBatchTileOptions; }

// Prices options [b, e) of the pool with the whole block: an unaligned head
// and tail one option per thread, the aligned body in groups of W options
// (W = 4: 16-byte loads, VPT = 2 groups per thread; W = 8: 256-bit loads,
// one group per thread).
template <int M, int W>
__device__ __forceinline__ void price_range(const SoA& pool, uint64_t b, uint64_t e) {
    constexpr uint64_t mask = W - 1;
    const uint64_t head_end = ((b + mask) & ~mask) < e ? ((b + mask) & ~mask) : e;
    const uint64_t body_end = (e & ~mask) > head_end ? (e & ~mask) : head_end;
    const uint64_t i_head = b + threadIdx.x;
    if (i_head < head_end) price_scalar<M>(pool, (int64_t)i_head);
    if constexpr (W == 8)
        price_groups<M, 8, 1, 2>(pool, (int64_t)(head_end / 8), (int64_t)(body_end / 8), 0ull, 0ull, 0);
    else
        price_groups<M, 4, kBatchVpt, 0>(pool, (int64_t)(head_end / 4), (int64_t)(body_end / 4), 0ull, 0ull, 0);
    const uint64_t i_tail = body_end + threadIdx.x;
    if (i_tail < e) price_scalar<M>(pool, (int64_t)i_tail);
}

// Persistent kernel: each block takes the next tile from the device work
// counter and prices it.  With a per-tile bounds table (tile_bounds[2 t],
// [2 t + 1] = the tile's [b, e) in the pool) a tile costs thread 0 one load;
// without it, a binary search over the tile prefix finds its segment.  The
// claim of the next tile is issued before the current one is priced, so the
// counter's round trip overlaps the pricing.  No block ever waits on another;
// the loop ends when the counter passes the last tile.  (Four blocks per SM
// hold the registers to 64; the libm mode's float-float exp/log get up to
// 128.)
template <int M, int W>
__global__ void __launch_bounds__(kBatchBlock, M == MODE_LIBM_REF ? 2 : 4) batch_kernel(
    SoA pool, const uint64_t* __restrict__ seg_off, const uint64_t* __restrict__ seg_len,
    const uint64_t* __restrict__ tile_prefix, const uint64_t* __restrict__ tile_bounds, int nseg,
    uint64_t ntiles, uint64_t topt, unsigned long long* cursor) {
    __shared__ uint64_t sh_b, sh_e;
    __shared__ int sh_done;
    pdl_trigger();
    unsigned long long next = 0;
    if (threadIdx.x == 0) next = atomicAdd(cursor, 1ull);
    for (;;) {
        if (threadIdx.x == 0) {
            const unsigned long long tile = next;
            if (tile >= ntiles) {
                sh_done = 1;
            } else {
                next = atomicAdd(cursor, 1ull);  // travels while this tile is priced
                if (tile_bounds) {
                    sh_b = tile_bounds[2 * tile];
                    sh_e = tile_bounds[2 * tile + 1];
                } else {
                    int lo = 0, hi = nseg - 1;
                    while (lo < hi) {  // largest segment whose first tile <= tile
                        const int mid = (lo + hi + 1) >> 1;
                        if (tile_prefix[mid] <= tile) lo = mid; else hi = mid - 1;
                    }
                    const uint64_t b = seg_off[lo] + (tile - tile_prefix[lo]) * topt;
                    const uint64_t send = seg_off[lo] + seg_len[lo];
                    sh_b = b;
                    sh_e = (b + topt < send) ? b + topt : send;
                }
                sh_done = 0;
            }
        }
        __syncthreads();
        const int done = sh_done;
        const uint64_t b = sh_b, e = sh_e;
        __syncthreads();
        if (done) break;
        price_range<M, W>(pool, b, e);
    }
    pdl_wait();
}

int batch_blocks_per_sm() {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_kernel<MODE_FAST, 8>, kBatchBlock, 0) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return n > 0 ? n : 1;
}

cudaError_t launch_batch(const SoA& pool, const uint64_t* seg_off,
                         const uint64_t* seg_len, const uint64_t* tile_prefix,
                         const uint64_t* tile_bounds, int nseg, uint64_t ntiles,
                         uint64_t tile_opts, unsigned long long* cursor, int mode, int grid,
                         int pdl, cudaStream_t st) {
    if (ntiles == 0 || nseg <= 0) return cudaSuccess;
    if (tile_opts == 0) return cudaErrorInvalidValue;
    if ((uint64_t)grid > ntiles) grid = (int)ntiles;  // no block without a tile
    if (grid < 1) grid = 1;
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)grid);
    lc.blockDim = dim3(kBatchBlock);
    lc.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    lc.attrs = attr;
    lc.numAttrs = pdl ? 1 : 0;
    // 256-bit loads need every pool array 32-byte aligned; the libm mode
    // keeps 128-bit loads (fewer registers: it is compute-bound)
    const bool w8 = mode != MODE_LIBM_REF && map_vectorizable(pool, MapCfg{1, kBatchBlock, 0, 2, 0});
#define BSG_BATCH(M_) \
    (w8 ? cudaLaunchKernelEx(&lc, batch_kernel<M_, 8>, pool, seg_off, seg_len, tile_prefix, \
                             tile_bounds, nseg, ntiles, tile_opts, cursor) \
        : cudaLaunchKernelEx(&lc, batch_kernel<M_, 4>, pool, seg_off, seg_len, tile_prefix, \
                             tile_bounds, nseg, ntiles, tile_opts, cursor))
    switch (mode) {
        case MODE_FAST: return BSG_BATCH(MODE_FAST);
        case MODE_SFU_REF: return BSG_BATCH(MODE_SFU_REF);
        case MODE_LIBM_REF: return BSG_BATCH(MODE_LIBM_REF);
        default: return cudaErrorInvalidValue;
    }
#undef BSG_BATCH
}

// ---------------------------------------------------------- error report
__global__ void __launch_bounds__(256) err_kernel(SoA a, const float* __restrict__ prices,
                                                  int64_t n, const double* __restrict__ edges,
                                                  int nb, double rel_floor, ErrAcc* acc) {
    __shared__ ErrAcc sh[kMaxErrBuckets];
    __shared__ double sh_edges[kMaxErrBuckets + 1];
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        sh[i].count = 0;
        sh[i].max_abs_bits = 0;
        sh[i].max_rel_bits = 0;
        sh[i].max_price_bits = 0;
        sh[i].sum_sq = 0.0;
    }
    for (int i = threadIdx.x; i <= nb; i += blockDim.x) sh_edges[i] = edges[i];
    __syncthreads();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double s = a.s[i], k = a.k[i], r = a.r[i], v = a.v[i], t = a.t[i];
        const double o = price_fp64(s, k, r, v, t, a.ot[i]);
        const double d1 = fabs(d1_fp64(s, k, r, v, t));
        int bk = 0;
        while (bk < nb - 1 && !(d1 < sh_edges[bk + 1])) ++bk;  // NaN -> last
        const double err = fabs((double)prices[i] - o);
        const double den = fabs(o) > rel_floor ? fabs(o) : rel_floor;
        const double rel = err / den;
        atomicAdd(&sh[bk].count, 1ull);
        atomicMax(&sh[bk].max_abs_bits, (unsigned long long)__double_as_longlong(err));
        atomicMax(&sh[bk].max_rel_bits, (unsigned long long)__double_as_longlong(rel));
        atomicMax(&sh[bk].max_price_bits, (unsigned long long)__double_as_longlong(fabs(o)));
        atomicAdd(&sh[bk].sum_sq, err * err);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        if (sh[i].count == 0) continue;
        atomicAdd(&acc[i].count, sh[i].count);
        atomicMax(&acc[i].max_abs_bits, sh[i].max_abs_bits);
        atomicMax(&acc[i].max_rel_bits, sh[i].max_rel_bits);
        atomicMax(&acc[i].max_price_bits, sh[i].max_price_bits);
        atomicAdd(&acc[i].sum_sq, sh[i].sum_sq);
    }
}

cudaError_t launch_err_report(const SoA& a, const float* prices, int64_t n,
                              const double* edges, int nbuckets, double rel_floor,
                              ErrAcc* acc, int sm_count, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (nbuckets < 1 || nbuckets > kMaxErrBuckets) return cudaErrorInvalidValue;
    int64_t grid = (n + 255) / 256;
    const int64_t cap = (int64_t)sm_count * 4;
    if (grid > cap) grid = cap;
    err_kernel<<<(unsigned)grid, 256, 0, st>>>(a, prices, n, edges, nbuckets, rel_floor, acc);
    return cudaGetLastError();
}

// -------------------------------------------------------------- fill (tuning)
__device__ __forceinline__ float hash_unit(uint64_t x) {
    x ^= x >> 33; x *= 0xff51afd7ed558ccdull; x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull; x ^= x >> 33;
    return (float)(x >> 40) * (1.0f / 16777216.0f);
}

__global__ void fill_kernel(SoA a, int64_t n, uint32_t seed) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t b = ((uint64_t)seed << 40) ^ ((uint64_t)i * 8);
        const float s = 10.0f + 190.0f * hash_unit(b + 1);
        float* ms = const_cast<float*>(a.s);
        float* mk = const_cast<float*>(a.k);
        float* mr = const_cast<float*>(a.r);
        float* mv = const_cast<float*>(a.v);
        float* mt = const_cast<float*>(a.t);
        int32_t* mo = const_cast<int32_t*>(a.ot);
        ms[i] = s;
        mk[i] = s * (0.5f + hash_unit(b + 2));
        mr[i] = 0.01f + 0.09f * hash_unit(b + 3);
        mv[i] = 0.05f + 0.6f * hash_unit(b + 4);
        mt[i] = 0.05f + 1.95f * hash_unit(b + 5);
        mo[i] = hash_unit(b + 6) < 0.5f ? 1 : 0;
    }
}

cudaError_t launch_fill(const SoA& a, int64_t n, uint32_t seed, int sm_count,
                        cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    int64_t grid = (n + 255) / 256;
    const int64_t cap = (int64_t)sm_count * 8;
    if (grid > cap) grid = cap;
    fill_kernel<<<(unsigned)grid, 256, 0, st>>>(a, n, seed);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Debug guards (contexts created with BSG_DEBUG set): one CTA row per array.

__global__ void guard_check_kernel(const uint32_t* __restrict__ base, int64_t stride,
                                   int64_t cap, int64_t out_lo, uint32_t pattern,
                                   unsigned long long* res) {
    const int64_t a = blockIdx.y;
    const int64_t lo = a == 6 ? out_lo : cap;
    unsigned long long cnt = 0, first = ~0ull;
    for (int64_t i = lo + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < stride;
         i += (int64_t)gridDim.x * blockDim.x) {
        if (base[a * stride + i] != pattern) {
            ++cnt;
            first = min(first, (unsigned long long)(a * stride + i));
        }
    }
    if (cnt) {
        atomicAdd(&res[0], cnt);
        atomicMin(&res[1], first);
    }
}

cudaError_t launch_guard_check(const uint32_t* base, int64_t stride, int64_t cap,
                               int64_t out_lo, uint32_t pattern, unsigned long long* res,
                               int sm_count, cudaStream_t st) {
    if (cap > stride || out_lo > stride || cap < 0 || out_lo < 0) return cudaErrorInvalidValue;
    const int64_t span = stride - (cap < out_lo ? cap : out_lo);
    int64_t gx = (span + 255) / 256;
    if (gx > 4LL * sm_count) gx = 4LL * sm_count;
    if (gx < 1) gx = 1;
    guard_check_kernel<<<dim3((unsigned)gx, 7), 256, 0, st>>>(base, stride, cap, out_lo,
                                                              pattern, res);
    return cudaGetLastError();
}

}  // namespace bsg
