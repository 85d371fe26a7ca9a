// bsg_noalloc.cu -- batched pricing for callers that cannot allocate memory.
//
// bsg_price_batch needs a context, and a context allocates device and pinned
// memory (resident buffers, the segment table, the tile counter).  Some
// callers cannot allow that: code running inside another runtime's memory
// pool or under a fixed device-memory budget, plugins loaded into a process
// that forbids new allocations after start-up, real-time loops where an
// allocation can block on the driver.  bsg_price_batch_noalloc prices the
// same books with no allocation at all: its scratch (the segment table, the
// per-segment tile prefix and the tile counter) lives in the fixed-size
// device array below, which every GPU that loads this library holds until
// the process exits.
//
// The scratch is shared by every call: a call overwrites the table and resets
// the counter, so calls must not overlap on the GPU (issue them on one stream
// or synchronise between them).  Overlapping calls get wrong prices; the
// kernel clamps every tile to its own pool so they never write outside it.
#include "bsg.h"
#include "bsg_internal.h"
#include "bsg_math.cuh"

#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

namespace {

constexpr int kMaxSeg = BSG_NOALLOC_MAX_SEGMENTS;
constexpr uint64_t kTile = 8192;     // options per tile
constexpr int kBlock = 256;
constexpr int kVpt = 2;              // v4 groups per thread per pass
constexpr int kHeader = 32;          // words: [0] tile counter, rest padding
// words: header | raw (offset,len) pairs | offsets | lengths | tile prefix
constexpr size_t kRaw = kHeader;
constexpr size_t kOff = kRaw + 2 * (size_t)kMaxSeg;
constexpr size_t kLen = kOff + kMaxSeg;
constexpr size_t kPre = kLen + kMaxSeg;
constexpr size_t kWords = kPre + kMaxSeg + 1;  // 20,513 words = 164,104 bytes

static __device__ __align__(256) unsigned long long bsg_noalloc_scratch[kWords];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
// The scratch array's device address per device, and the driver context it
// was looked up in: after a device reset the module loads again in a new
// context and the array may sit elsewhere, so a changed context id means
// the address is looked up again.
unsigned long long* g_addr[kMaxDevices];
unsigned long long g_ctx_id[kMaxDevices];

// Builds the table from the raw pairs the host copied in: de-interleaves the
// pairs, writes each segment's first tile (exclusive prefix of
// ceil(len / kTile)) and zeroes the tile counter.  One block of 1024 threads.
__global__ void __launch_bounds__(1024) noalloc_setup_kernel(unsigned long long* scratch, int nseg) {
    __shared__ unsigned long long part[1024];
    const unsigned long long* raw = scratch + kRaw;
    unsigned long long* off = scratch + kOff;
    unsigned long long* len = scratch + kLen;
    unsigned long long* pre = scratch + kPre;
    const int per = (nseg + 1023) / 1024;
    const int i0 = threadIdx.x * per;
    const int i1 = min(i0 + per, nseg);
    unsigned long long sum = 0;
    for (int i = i0; i < i1; ++i) {
        const unsigned long long o = raw[2 * i], l = raw[2 * i + 1];
        off[i] = o;
        len[i] = l;
        sum += (l + kTile - 1) / kTile;
    }
    part[threadIdx.x] = sum;
    __syncthreads();
    for (int d = 1; d < 1024; d <<= 1) {  // inclusive scan (Hillis-Steele)
        const unsigned long long x = threadIdx.x >= d ? part[threadIdx.x - d] : 0ull;
        __syncthreads();
        part[threadIdx.x] += x;
        __syncthreads();
    }
    unsigned long long acc = part[threadIdx.x] - sum;  // exclusive
    for (int i = i0; i < i1; ++i) {
        pre[i] = acc;
        acc += (len[i] + kTile - 1) / kTile;
    }
    if (threadIdx.x == 1023) pre[nseg] = part[1023];
    if (threadIdx.x == 0) scratch[0] = 0ull;
}

__device__ __forceinline__ void price_one(const bsg::SoA& p, uint64_t i) {
    p.out[i] = bsg::price<bsg::MODE_FAST>(__ldg(p.s + i), __ldg(p.k + i), __ldg(p.r + i),
                                         __ldg(p.v + i), __ldg(p.t + i), __ldg(p.ot + i));
}

// Options [b, e) with the whole block: unaligned head and tail one option per
// thread, the 16-byte aligned body as float4 groups, kVpt per thread per pass.
__device__ __forceinline__ void price_tile(const bsg::SoA& p, uint64_t b, uint64_t e) {
    const uint64_t head_end = ((b + 3) & ~3ull) < e ? ((b + 3) & ~3ull) : e;
    const uint64_t body_end = (e & ~3ull) > head_end ? (e & ~3ull) : head_end;
    if (b + threadIdx.x < head_end) price_one(p, b + threadIdx.x);
    const uint64_t g0 = head_end / 4, g1 = body_end / 4;
    for (uint64_t base = g0; base < g1; base += (uint64_t)kBlock * kVpt) {
        float4 S[kVpt], K[kVpt], R[kVpt], V[kVpt], T[kVpt];
        int4 O[kVpt];
#pragma unroll
        for (int j = 0; j < kVpt; ++j) {
            const uint64_t g = base + threadIdx.x + (uint64_t)j * kBlock;
            if (g < g1) {
                S[j] = __ldg(reinterpret_cast<const float4*>(p.s) + g);
                K[j] = __ldg(reinterpret_cast<const float4*>(p.k) + g);
                R[j] = __ldg(reinterpret_cast<const float4*>(p.r) + g);
                V[j] = __ldg(reinterpret_cast<const float4*>(p.v) + g);
                T[j] = __ldg(reinterpret_cast<const float4*>(p.t) + g);
                O[j] = __ldg(reinterpret_cast<const int4*>(p.ot) + g);
            }
        }
#pragma unroll
        for (int j = 0; j < kVpt; ++j) {
            const uint64_t g = base + threadIdx.x + (uint64_t)j * kBlock;
            if (g < g1) {
                float4 q;
                q.x = bsg::price<bsg::MODE_FAST>(S[j].x, K[j].x, R[j].x, V[j].x, T[j].x, O[j].x);
                q.y = bsg::price<bsg::MODE_FAST>(S[j].y, K[j].y, R[j].y, V[j].y, T[j].y, O[j].y);
                q.z = bsg::price<bsg::MODE_FAST>(S[j].z, K[j].z, R[j].z, V[j].z, T[j].z, O[j].z);
                q.w = bsg::price<bsg::MODE_FAST>(S[j].w, K[j].w, R[j].w, V[j].w, T[j].w, O[j].w);
                __stcs(reinterpret_cast<float4*>(p.out) + g, q);
            }
        }
    }
    if (body_end + threadIdx.x < e) price_one(p, body_end + threadIdx.x);
}

// Persistent kernel over the scratch table: blocks take tiles from the
// counter in scratch[0] until it passes ntiles.  Every tile is clamped to
// [0, pool_len), so a table left by another call can never lead a block
// outside this call's pool.
__global__ void __launch_bounds__(kBlock) noalloc_batch_kernel(
    bsg::SoA pool, uint64_t pool_len, unsigned long long* scratch, int nseg, uint64_t ntiles) {
    __shared__ uint64_t sh_b, sh_e;
    __shared__ int sh_done;
    const unsigned long long* off = scratch + kOff;
    const unsigned long long* len = scratch + kLen;
    const unsigned long long* pre = scratch + kPre;
    for (;;) {
        if (threadIdx.x == 0) {
            const unsigned long long tile = atomicAdd(&scratch[0], 1ull);
            sh_done = tile >= ntiles;
            if (!sh_done) {
                int lo = 0, hi = nseg - 1;
                while (lo < hi) {  // largest segment whose first tile <= tile
                    const int mid = (lo + hi + 1) >> 1;
                    if (pre[mid] <= tile) lo = mid; else hi = mid - 1;
                }
                uint64_t b = off[lo] + (tile - pre[lo]) * kTile;
                uint64_t e = off[lo] + len[lo];
                e = (b + kTile < e) ? b + kTile : e;
                e = e < pool_len ? e : pool_len;
                b = b < e ? b : e;
                sh_b = b;
                sh_e = e;
            }
        }
        __syncthreads();
        const int done = sh_done;
        const uint64_t b = sh_b, e = sh_e;
        __syncthreads();
        if (done) break;
        if (b < e) price_tile(pool, b, e);
    }
}

// [p, p + bytes) device memory of `device` (one allocation, or consecutive
// mapped pieces of a virtual range), 16-byte aligned.
bool dev_range_ok(const void* p, size_t bytes, int device) {
    if (!p || (reinterpret_cast<uintptr_t>(p) & 15)) return false;
    return bsg::device_extent(p, bytes, device) == bsg::kExtentOk;
}

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

template <typename Fn>
Fn driver_fn(const char* name) {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion(name, &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return reinterpret_cast<Fn>(f);
}

// The unique id of the calling thread's current driver context (0 if none
// or unknown).  The runtime calls above have made the primary context of
// the current device current.
unsigned long long current_ctx_id() {
    static CtxGetCurrentFn get_cur = driver_fn<CtxGetCurrentFn>("cuCtxGetCurrent");
    static CtxGetIdFn get_id = driver_fn<CtxGetIdFn>("cuCtxGetId");
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!get_cur || !get_id || get_cur(&ctx) != CUDA_SUCCESS || !ctx ||
        get_id(ctx, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}

}  // namespace

extern "C" int bsg_price_batch_noalloc(const float* sptprice, const float* strike,
                                       const float* rate, const float* volatility,
                                       const float* otime, const int32_t* otype,
                                       float* prices, size_t pool_len,
                                       const bsg_segment* segs, size_t nseg, void* stream,
                                       unsigned flags) {
    if ((flags & ~(BSG_DEVICE_PTRS | BSG_ASYNC)) != 0) return BSG_ERR_INVALID_ARG;
    if (nseg > (size_t)kMaxSeg) return BSG_ERR_CAPACITY;  // scratch holds kMaxSeg segments
    if (nseg && !segs) return BSG_ERR_INVALID_ARG;
    if (pool_len == 0 || nseg == 0) return BSG_OK;
    if (pool_len > ((size_t)1 << 36)) return BSG_ERR_INVALID_ARG;
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices) {
        cudaGetLastError();
        return BSG_ERR_NO_DEVICE;
    }
    const size_t bytes = pool_len * 4;
    if (!dev_range_ok(sptprice, bytes, device) || !dev_range_ok(strike, bytes, device) ||
        !dev_range_ok(rate, bytes, device) || !dev_range_ok(volatility, bytes, device) ||
        !dev_range_ok(otime, bytes, device) || !dev_range_ok(otype, bytes, device) ||
        !dev_range_ok(prices, bytes, device))
        return BSG_ERR_INVALID_ARG;
    uint64_t ntiles = 0;
    for (size_t i = 0; i < nseg; ++i) {
        const uint64_t o = segs[i].offset, l = segs[i].len;
        if (o > pool_len || l > pool_len - o) return BSG_ERR_INVALID_ARG;
        ntiles += (l + kTile - 1) / kTile;
    }
    if (ntiles == 0) return BSG_OK;

    // Set-up, once per device (and again after a device reset) with that
    // device current: the device address of the scratch array (its
    // host-side name is only a stand-in).
    unsigned long long* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        const unsigned long long ctx_id = current_ctx_id();
        if (!g_addr[device] || ctx_id == 0 || ctx_id != g_ctx_id[device]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, bsg_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                cudaGetLastError();
                g_addr[device] = nullptr;
                return BSG_ERR_CUDA;
            }
            g_addr[device] = static_cast<unsigned long long*>(p);
            g_ctx_id[device] = ctx_id;
        }
        scratch = g_addr[device];
    }
    int sms = 0, bps = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, noalloc_batch_kernel, kBlock, 0) !=
            cudaSuccess) {
        cudaGetLastError();
        return BSG_ERR_CUDA;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaMemcpyAsync(scratch + kRaw, segs, nseg * sizeof(bsg_segment), cudaMemcpyHostToDevice,
                        st) != cudaSuccess) {
        cudaGetLastError();
        return BSG_ERR_CUDA;
    }
    noalloc_setup_kernel<<<1, 1024, 0, st>>>(scratch, (int)nseg);
    bsg::SoA pool{sptprice, strike, rate, volatility, otime, otype, prices};
    noalloc_batch_kernel<<<sms * (bps > 0 ? bps : 1), kBlock, 0, st>>>(pool, pool_len, scratch,
                                                                       (int)nseg, ntiles);
    if (cudaGetLastError() != cudaSuccess) return BSG_ERR_CUDA;
    if (!(flags & BSG_ASYNC) && cudaStreamSynchronize(st) != cudaSuccess) {
        cudaGetLastError();
        return BSG_ERR_CUDA;
    }
    return BSG_OK;
}
