// bsg_api.cu -- the C ABI of libbsgpu.so (declared in include/bsg.h).
//
// A context owns a device, a stream, resident buffers for host-pointer calls,
// a small cache of instantiated CUDA graphs (the NUM_RUNS loop replayed as
// one graph launch), device scratch for batch segment tables and error
// accumulators, and the tuning choice of the plain map.
//
// Safety: every device pointer handed in is checked against the extent of
// the allocation that contains it (cuMemGetAddressRange) before any kernel
// reads or writes through it, so a wrong size or pointer from the caller is
// a status code, never an out-of-bounds access on the GPU.
#include "bsg.h"
#include "bsg_internal.h"

#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <mutex>
#include <new>
#include <sstream>
#include <string>
#include <vector>

namespace {

constexpr size_t kGraphCacheSize = 8;

struct GraphKey {
    bsg::SoA soa;
    int64_t n;
    int runs;
    int mode;
    bsg::MapCfg cfg;
    int kind;  // 0 plain map, 1 batch
    uint64_t ntiles;
    int nseg;
    uint64_t btile;  // batch tile (options) and grid
    int bgrid;
    bool operator==(const GraphKey& o) const {
        return std::memcmp(this, &o, sizeof(GraphKey)) == 0;
    }
};

struct GraphEntry {
    GraphKey key;
    cudaGraphExec_t exec;
};

// Flag bits the map entry points accept.
constexpr unsigned kMapFlags = BSG_DEVICE_PTRS | BSG_ASYNC | BSG_MODE_MASK | BSG_NO_GRAPH;

int mode_of(unsigned flags) {
    if (flags & ~kMapFlags) return -1;
    switch (flags & BSG_MODE_MASK) {
        case BSG_MODE_FAST: return bsg::MODE_FAST;
        case BSG_MODE_SFU_REF: return bsg::MODE_SFU_REF;
        case BSG_MODE_LIBM_REF: return bsg::MODE_LIBM_REF;
        default: return -1;
    }
}

size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

constexpr size_t kGuardWords = 64;        // guard words after each resident array
constexpr int kGuardByte = 0xA5;          // guard fill byte
constexpr uint32_t kGuardWord = 0xA5A5A5A5u;

bool debug_env() {
    const char* e = std::getenv("BSG_DEBUG");
    return e && *e && std::strcmp(e, "0") != 0;
}

}  // namespace

struct bsg_ctx {
    int device = 0;
    int sm_count = 0;
    int batch_blocks_per_sm = 1;  // occupancy limit of the batch kernel
    uint64_t batch_tile = 8192;   // batch tuning (bsg_autotune_batch)
    int batch_bps = 0;            // 0 = the occupancy limit
    cudaStream_t stream = nullptr;
    size_t cap = 0;     // max_options
    size_t cap_al = 0;  // per-array stride in the resident buffer
    char* dev_buf = nullptr;
    bsg::MapCfg tune{1, 256, 0, 0, 0};
    std::mutex mu;
    std::string err;
    uint64_t launches = 0;
    std::vector<GraphEntry> graphs;
    // batch scratch: [off | len | prefix] of seg_cap (+1) entries
    uint64_t* d_seg = nullptr;
    size_t seg_cap = 0;
    uint64_t* h_seg = nullptr;  // pinned staging of the same layout
    // per-tile [begin, end) of the batch (2 entries per tile), device and
    // pinned staging
    uint64_t* d_tb = nullptr;
    uint64_t* h_tb = nullptr;
    size_t tb_cap = 0;  // tiles
    cudaEvent_t seg_ev = nullptr;
    unsigned long long* d_cursor = nullptr;  // one work counter per pass
    size_t cursor_cap = 0;
    // error-report scratch
    bsg::ErrAcc* d_acc = nullptr;
    double* d_edges = nullptr;
    // pipelined host calls (BSG_ASYNC with host pointers): a second resident
    // set, copy-in and copy-out streams, and per-set events
    char* dev_buf2 = nullptr;
    cudaStream_t copy_in = nullptr, copy_out = nullptr;
    cudaEvent_t ev_in[2] = {nullptr, nullptr};
    cudaEvent_t ev_comp[2] = {nullptr, nullptr};
    cudaEvent_t ev_out[2] = {nullptr, nullptr};
    int next_set = 0;
    bool pipelined = false;  // pipelined work may be in flight
    // debug guards (BSG_DEBUG set at bsg_create): every resident array is
    // followed by at least kGuardWords words of kGuardByte, checked after
    // each synchronous call; d_guard holds the check's {count, first index}
    bool debug = false;
    unsigned long long* d_guard = nullptr;
    // swaption scratch: parameter table, per-block partial sums, results
    char* d_sw = nullptr;
    size_t sw_cap = 0;

    bsg::SoA resident(size_t n, int set = 0) const {
        (void)n;
        float* f = reinterpret_cast<float*>(set ? dev_buf2 : dev_buf);
        bsg::SoA a;
        a.s = f;
        a.k = f + cap_al;
        a.r = f + 2 * cap_al;
        a.v = f + 3 * cap_al;
        a.t = f + 4 * cap_al;
        a.ot = reinterpret_cast<const int32_t*>(f + 5 * cap_al);
        a.out = f + 6 * cap_al;
        return a;
    }
};

namespace {

int fail(bsg_ctx* c, int st, const std::string& msg) {
    if (c) c->err = msg;
    return st;
}

int cuda_fail(bsg_ctx* c, cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    if (e == cudaErrorMemoryAllocation) return fail(c, BSG_ERR_OUT_OF_MEMORY, m);
    return fail(c, BSG_ERR_CUDA, m);
}

#define BSG_CK(c, call)                                  \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return cuda_fail(c, e_, #call); \
    } while (0)

// cuMemGetAddressRange, resolved through the runtime so that the library has
// no link-time dependency on libcuda (it loads on machines without a driver).
typedef CUresult (*MemGetAddressRangeFn)(CUdeviceptr*, size_t*, CUdeviceptr);

MemGetAddressRangeFn mem_get_address_range() {
    static MemGetAddressRangeFn fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuMemGetAddressRange", &f, 12000,
                                             cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            f = nullptr;
        }
        return reinterpret_cast<MemGetAddressRangeFn>(f);
    }();
    return fn;
}

typedef CUresult (*PointerGetAttributeFn)(void*, CUpointer_attribute, CUdeviceptr);
typedef CUresult (*MemGetAccessFn)(unsigned long long*, const CUmemLocation*, CUdeviceptr);

template <typename Fn>
Fn driver_entry(const char* name) {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion(name, &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return reinterpret_cast<Fn>(f);
}

// Whether the mapped piece at p was mapped through the virtual memory API
// (cuMemCreate + cuMemMap: not usable with legacy IPC, unlike cudaMalloc
// memory) and gives `device` read-write access.
bool vmm_piece_rw(uintptr_t p, int device) {
    static PointerGetAttributeFn get_attr =
        driver_entry<PointerGetAttributeFn>("cuPointerGetAttribute");
    static MemGetAccessFn get_access = driver_entry<MemGetAccessFn>("cuMemGetAccess");
    if (!get_attr || !get_access) return false;
    unsigned long long legacy_ipc = 0;  // a boolean: zero-filled whatever its width
    if (get_attr(&legacy_ipc, CU_POINTER_ATTRIBUTE_IS_LEGACY_CUDA_IPC_CAPABLE, (CUdeviceptr)p) !=
            CUDA_SUCCESS ||
        legacy_ipc != 0)
        return false;
    CUmemLocation loc;
    loc.type = CU_MEM_LOCATION_TYPE_DEVICE;
    loc.id = device;
    unsigned long long flags = 0;
    return get_access(&flags, &loc, (CUdeviceptr)p) == CUDA_SUCCESS &&
           flags == CU_MEM_ACCESS_FLAGS_PROT_READWRITE;
}

}  // namespace

namespace bsg {

int device_extent(const void* p, size_t bytes, int device) {
    const uintptr_t want = reinterpret_cast<uintptr_t>(p) + bytes;
    if (want < reinterpret_cast<uintptr_t>(p)) return kExtentOverrun;
    MemGetAddressRangeFn range = mem_get_address_range();
    if (!range) return kExtentUnknown;
    uintptr_t cur = reinterpret_cast<uintptr_t>(p);
    for (int piece = 0; piece < 65536; ++piece) {
        cudaPointerAttributes attr;
        if (cudaPointerGetAttributes(&attr, reinterpret_cast<const void*>(cur)) != cudaSuccess) {
            cudaGetLastError();
            return piece ? kExtentOverrun : kExtentNotDevice;
        }
        if (attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged)
            return piece ? kExtentOverrun : kExtentNotDevice;
        if (attr.type == cudaMemoryTypeDevice && attr.device != device)
            return piece ? kExtentOverrun : kExtentOtherDevice;
        CUdeviceptr base = 0;
        size_t size = 0;
        if (range(&base, &size, (CUdeviceptr)cur) != CUDA_SUCCESS)
            return piece ? kExtentOverrun : kExtentUnknown;
        const uintptr_t end = (uintptr_t)base + size;
        // a piece of a virtual range must itself be readable and writable
        // by the device; one cudaMalloc allocation is
        const bool vmm = attr.type == cudaMemoryTypeDevice && vmm_piece_rw(cur, device);
        if (piece && !vmm) return kExtentOverrun;
        if (want <= end) return kExtentOk;
        // past this piece: go on only from one mapped piece of a virtual
        // range to the next, never from one ordinary allocation to another
        if (!vmm) return kExtentOverrun;
        cur = end;
    }
    return kExtentOverrun;
}

}  // namespace bsg

namespace {

// Checks that [p, p + bytes) is device memory of the context's device:
// inside one allocation, or across consecutive mapped pieces of a virtual
// range (bsg::device_extent).
int check_dev_range(bsg_ctx* c, const void* p, size_t bytes, const char* name) {
    if (!p) return fail(c, BSG_ERR_INVALID_ARG, std::string(name) + " is NULL");
    if ((reinterpret_cast<uintptr_t>(p) & 3) != 0)
        return fail(c, BSG_ERR_MISALIGNED, std::string(name) + " is not 4-byte aligned");
    switch (bsg::device_extent(p, bytes, c->device)) {
        case bsg::kExtentOk: return BSG_OK;
        case bsg::kExtentNotDevice:
            return fail(c, BSG_ERR_INVALID_ARG, std::string(name) + " is not device memory");
        case bsg::kExtentOtherDevice:
            return fail(c, BSG_ERR_INVALID_ARG, std::string(name) + " lives on another device");
        case bsg::kExtentUnknown:
            return fail(c, BSG_ERR_INVALID_ARG, std::string(name) + ": allocation range unknown");
        default:
            return fail(c, BSG_ERR_INVALID_ARG,
                        std::string(name) + ": " + std::to_string(bytes) +
                            " bytes run past the end of its allocation");
    }
}

int check_soa_dev(bsg_ctx* c, const bsg::SoA& a, size_t n, size_t out_elem) {
    const size_t b = n * 4;
    int st;
    if ((st = check_dev_range(c, a.s, b, "sptprice"))) return st;
    if ((st = check_dev_range(c, a.k, b, "strike"))) return st;
    if ((st = check_dev_range(c, a.r, b, "rate"))) return st;
    if ((st = check_dev_range(c, a.v, b, "volatility"))) return st;
    if ((st = check_dev_range(c, a.t, b, "otime"))) return st;
    if ((st = check_dev_range(c, a.ot, b, "otype"))) return st;
    if (out_elem && (st = check_dev_range(c, a.out, n * out_elem, "prices"))) return st;
    return BSG_OK;
}

int check_soa_host(bsg_ctx* c, const bsg::SoA& a) {
    if (!a.s || !a.k || !a.r || !a.v || !a.t || !a.ot || !a.out)
        return fail(c, BSG_ERR_INVALID_ARG, "a host array is NULL");
    return BSG_OK;
}

void graph_drop_all(bsg_ctx* c) {
    for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
    c->graphs.clear();
}

cudaGraphExec_t graph_find(bsg_ctx* c, const GraphKey& k) {
    for (size_t i = 0; i < c->graphs.size(); ++i) {
        if (c->graphs[i].key == k) {
            GraphEntry e = c->graphs[i];  // move to front (LRU)
            c->graphs.erase(c->graphs.begin() + i);
            c->graphs.insert(c->graphs.begin(), e);
            return e.exec;
        }
    }
    return nullptr;
}

void graph_put(bsg_ctx* c, const GraphKey& k, cudaGraphExec_t exec) {
    if (c->graphs.size() >= kGraphCacheSize) {
        cudaGraphExecDestroy(c->graphs.back().exec);
        c->graphs.pop_back();
    }
    c->graphs.insert(c->graphs.begin(), GraphEntry{k, exec});
}

GraphKey make_key(const bsg::SoA& a, int64_t n, int runs, int mode,
                  const bsg::MapCfg& cfg, int kind, uint64_t ntiles, int nseg,
                  uint64_t btile = 0, int bgrid = 0) {
    GraphKey k;
    std::memset(static_cast<void*>(&k), 0, sizeof(k));  // padding must compare equal
    k.soa = a;
    k.n = n;
    k.runs = runs;
    k.mode = mode;
    k.cfg = cfg;
    k.kind = kind;
    k.ntiles = ntiles;
    k.nseg = nseg;
    k.btile = btile;
    k.bgrid = bgrid;
    return k;
}

// Enqueues `runs` passes of the plain map on the context stream, from a
// cached graph when runs > 1 and graphs are allowed.
int enqueue_map_runs(bsg_ctx* c, const bsg::SoA& a, int64_t n, int runs, int mode,
                     unsigned flags) {
    if (n <= 0 || runs <= 0) return BSG_OK;
    const bsg::MapCfg cfg = c->tune;
    if (runs == 1 || (flags & BSG_NO_GRAPH)) {
        for (int j = 0; j < runs; ++j) {
            cudaError_t e = bsg::launch_map(a, n, mode, bsg::pass_cfg(cfg, j, runs), c->sm_count,
                                            c->stream);
            if (e != cudaSuccess) return cuda_fail(c, e, "launch_map");
            c->launches++;
        }
        return BSG_OK;
    }
    GraphKey key = make_key(a, n, runs, mode, cfg, 0, 0, 0);
    cudaGraphExec_t exec = graph_find(c, key);
    if (!exec) {
        cudaGraph_t g = nullptr;
        BSG_CK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t le = cudaSuccess;
        for (int j = 0; j < runs && le == cudaSuccess; ++j)
            le = bsg::launch_map(a, n, mode, bsg::pass_cfg(cfg, j, runs), c->sm_count, c->stream);
        cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
        if (le != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return cuda_fail(c, le, "launch_map (capture)");
        }
        if (ce != cudaSuccess) return cuda_fail(c, ce, "cudaStreamEndCapture");
        cudaError_t ie = cudaGraphInstantiate(&exec, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) return cuda_fail(c, ie, "cudaGraphInstantiate");
        graph_put(c, key, exec);
    }
    BSG_CK(c, cudaGraphLaunch(exec, c->stream));
    c->launches += (uint64_t)runs;
    return BSG_OK;
}

// The bulk-staged kernel reports an expired wait in an error word; any call
// that synchronises checks it.
int check_bulk_error(bsg_ctx* c) {
    if (c->tune.load_path >= 3 && c->tune.load_path <= 5 && bsg::bulk_error_take())
        return fail(c, BSG_ERR_TIMEOUT, "a bulk-copy wait of the staged map kernel expired");
    return BSG_OK;
}

// Debug guards: checks that the guard words of both resident sets still hold
// the fill (set 0's price array from out_lo on, every other array from
// max_options on) once the context's streams are idle.  A difference means a
// kernel or a copy wrote past the options it was given: BSG_ERR_STATE, with
// the first overwritten word.
int debug_check(bsg_ctx* c, size_t out_lo) {
    if (!c->debug) return BSG_OK;
    for (int set = 0; set < 2; ++set) {
        const char* buf = set ? c->dev_buf2 : c->dev_buf;
        if (!buf) continue;
        BSG_CK(c, cudaMemsetAsync(c->d_guard, 0, 8, c->stream));
        BSG_CK(c, cudaMemsetAsync(c->d_guard + 1, 0xFF, 8, c->stream));
        cudaError_t e = bsg::launch_guard_check(
            reinterpret_cast<const uint32_t*>(buf), (int64_t)c->cap_al, (int64_t)c->cap,
            (int64_t)(set ? c->cap : out_lo), kGuardWord, c->d_guard, c->sm_count, c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "launch_guard_check");
        c->launches++;
        unsigned long long h[2] = {0, 0};
        BSG_CK(c, cudaMemcpyAsync(h, c->d_guard, sizeof h, cudaMemcpyDeviceToHost, c->stream));
        BSG_CK(c, cudaStreamSynchronize(c->stream));
        if (h[0]) {
            static const char* names[7] = {"sptprice", "strike", "rate", "volatility",
                                           "otime", "otype", "prices"};
            const size_t arr = (size_t)(h[1] / c->cap_al), off = (size_t)(h[1] % c->cap_al);
            return fail(c, BSG_ERR_STATE,
                        "debug guard: " + std::to_string(h[0]) +
                            " guard word(s) overwritten in resident set " + std::to_string(set) +
                            "; first: " + names[arr < 7 ? arr : 6] + "[" + std::to_string(off) +
                            "] (max_options " + std::to_string(c->cap) + ")");
        }
    }
    return BSG_OK;
}

// Debug guards: refills set 0's price array from n on before a synchronous
// host call of n options, so that the check after it covers [n, max_options).
int debug_arm(bsg_ctx* c, size_t n) {
    if (!c->debug) return BSG_OK;
    float* out = reinterpret_cast<float*>(c->dev_buf) + 6 * c->cap_al;
    BSG_CK(c, cudaMemsetAsync(out + n, kGuardByte, (c->cap_al - n) * 4, c->stream));
    return BSG_OK;
}

int finish(bsg_ctx* c, unsigned flags) {
    if (flags & BSG_ASYNC) return BSG_OK;
    BSG_CK(c, cudaStreamSynchronize(c->stream));
    int st = check_bulk_error(c);
    return st ? st : debug_check(c, c->cap);
}

// Waits for pipelined host calls (all three streams).
int drain_pipeline(bsg_ctx* c) {
    if (!c->pipelined) return BSG_OK;
    BSG_CK(c, cudaStreamSynchronize(c->copy_in));
    BSG_CK(c, cudaStreamSynchronize(c->stream));
    BSG_CK(c, cudaStreamSynchronize(c->copy_out));
    c->pipelined = false;
    int st = check_bulk_error(c);
    return st ? st : debug_check(c, c->cap);
}

int ensure_pipeline(bsg_ctx* c) {
    if (c->dev_buf2) return BSG_OK;
    BSG_CK(c, cudaStreamCreateWithFlags(&c->copy_in, cudaStreamNonBlocking));
    BSG_CK(c, cudaStreamCreateWithFlags(&c->copy_out, cudaStreamNonBlocking));
    for (int b = 0; b < 2; ++b) {
        BSG_CK(c, cudaEventCreateWithFlags(&c->ev_in[b], cudaEventDisableTiming));
        BSG_CK(c, cudaEventCreateWithFlags(&c->ev_comp[b], cudaEventDisableTiming));
        BSG_CK(c, cudaEventCreateWithFlags(&c->ev_out[b], cudaEventDisableTiming));
    }
    BSG_CK(c, cudaMalloc(&c->dev_buf2, 7 * c->cap_al * sizeof(float)));
    if (c->debug) {
        // the copy-in stream writes this set next: fill it before returning
        BSG_CK(c, cudaMemsetAsync(c->dev_buf2, kGuardByte, 7 * c->cap_al * sizeof(float), c->stream));
        BSG_CK(c, cudaStreamSynchronize(c->stream));
    }
    return BSG_OK;
}

// A pipelined host call: inputs copied into the next of two resident sets on
// the copy-in stream, the passes on the compute stream, prices copied out on
// the copy-out stream; events order each set's reuse.  Successive calls
// overlap one call's copies with another's passes.
int enqueue_host_pipelined(bsg_ctx* c, const bsg::SoA& h, size_t n, int runs, int mode,
                           unsigned flags) {
    int st;
    if ((st = ensure_pipeline(c))) return st;
    const int b = c->next_set;
    c->next_set ^= 1;
    const bsg::SoA d = c->resident(n, b);
    const size_t by = n * 4;
    // this set's inputs may be overwritten once its previous passes are done
    BSG_CK(c, cudaStreamWaitEvent(c->copy_in, c->ev_comp[b], 0));
    BSG_CK(c, cudaMemcpyAsync((void*)d.s, h.s, by, cudaMemcpyHostToDevice, c->copy_in));
    BSG_CK(c, cudaMemcpyAsync((void*)d.k, h.k, by, cudaMemcpyHostToDevice, c->copy_in));
    BSG_CK(c, cudaMemcpyAsync((void*)d.r, h.r, by, cudaMemcpyHostToDevice, c->copy_in));
    BSG_CK(c, cudaMemcpyAsync((void*)d.v, h.v, by, cudaMemcpyHostToDevice, c->copy_in));
    BSG_CK(c, cudaMemcpyAsync((void*)d.t, h.t, by, cudaMemcpyHostToDevice, c->copy_in));
    BSG_CK(c, cudaMemcpyAsync((void*)d.ot, h.ot, by, cudaMemcpyHostToDevice, c->copy_in));
    BSG_CK(c, cudaEventRecord(c->ev_in[b], c->copy_in));
    // the passes need the inputs, and this set's previous prices read out
    BSG_CK(c, cudaStreamWaitEvent(c->stream, c->ev_in[b], 0));
    BSG_CK(c, cudaStreamWaitEvent(c->stream, c->ev_out[b], 0));
    c->pipelined = true;
    if ((st = enqueue_map_runs(c, d, (int64_t)n, runs, mode, flags))) return st;
    BSG_CK(c, cudaEventRecord(c->ev_comp[b], c->stream));
    BSG_CK(c, cudaStreamWaitEvent(c->copy_out, c->ev_comp[b], 0));
    BSG_CK(c, cudaMemcpyAsync(h.out, d.out, by, cudaMemcpyDeviceToHost, c->copy_out));
    BSG_CK(c, cudaEventRecord(c->ev_out[b], c->copy_out));
    return BSG_OK;
}

int grow_seg_scratch(bsg_ctx* c, size_t nseg) {
    if (nseg <= c->seg_cap) return BSG_OK;
    size_t cap = std::max<size_t>(nseg, 1024);
    cap = round_up(cap, 1024);
    if (c->seg_ev) BSG_CK(c, cudaEventSynchronize(c->seg_ev));
    BSG_CK(c, cudaStreamSynchronize(c->stream));
    graph_drop_all(c);  // graphs hold the old table address
    if (c->d_seg) cudaFree(c->d_seg);
    if (c->h_seg) cudaFreeHost(c->h_seg);
    c->d_seg = nullptr;
    c->h_seg = nullptr;
    c->seg_cap = 0;
    BSG_CK(c, cudaMalloc(&c->d_seg, (3 * cap + 1) * sizeof(uint64_t)));
    BSG_CK(c, cudaMallocHost(&c->h_seg, (3 * cap + 1) * sizeof(uint64_t)));
    c->seg_cap = cap;
    return BSG_OK;
}

int grow_tile_scratch(bsg_ctx* c, size_t ntiles) {
    if (ntiles <= c->tb_cap) return BSG_OK;
    const size_t cap = round_up(std::max<size_t>(ntiles, 4096), 4096);
    if (c->seg_ev) BSG_CK(c, cudaEventSynchronize(c->seg_ev));
    BSG_CK(c, cudaStreamSynchronize(c->stream));
    graph_drop_all(c);  // graphs hold the old table address
    if (c->d_tb) cudaFree(c->d_tb);
    if (c->h_tb) cudaFreeHost(c->h_tb);
    c->d_tb = nullptr;
    c->h_tb = nullptr;
    c->tb_cap = 0;
    BSG_CK(c, cudaMalloc(&c->d_tb, 2 * cap * sizeof(uint64_t)));
    BSG_CK(c, cudaMallocHost(&c->h_tb, 2 * cap * sizeof(uint64_t)));
    c->tb_cap = cap;
    return BSG_OK;
}

// Validates the segments and writes the compacted (non-empty) table, and
// every tile's [begin, end), into the pinned staging buffers.  Returns the
// count of non-empty segments.
int build_segments(bsg_ctx* c, const bsg_segment* segs, size_t nseg, size_t pool_len,
                   uint64_t tile, int* nseg_out, uint64_t* ntiles_out) {
    std::vector<std::pair<uint64_t, uint64_t>> v;
    v.reserve(nseg);
    for (size_t i = 0; i < nseg; ++i) {
        const uint64_t o = segs[i].offset, l = segs[i].len;
        if (o > pool_len || l > pool_len - o)
            return fail(c, BSG_ERR_INVALID_ARG, "segment " + std::to_string(i) + " lies outside the pool");
        if (l) v.emplace_back(o, l);
    }
    std::vector<std::pair<uint64_t, uint64_t>> sorted(v);
    std::sort(sorted.begin(), sorted.end());
    for (size_t i = 1; i < sorted.size(); ++i)
        if (sorted[i - 1].first + sorted[i - 1].second > sorted[i].first)
            return fail(c, BSG_ERR_INVALID_ARG, "segments overlap");
    if (v.size() > 0x7fffffff) return fail(c, BSG_ERR_INVALID_ARG, "too many segments");
    int st = grow_seg_scratch(c, v.size());
    if (st) return st;
    if (c->seg_ev) BSG_CK(c, cudaEventSynchronize(c->seg_ev));  // staging reuse
    const size_t m = v.size();
    uint64_t* off = c->h_seg;
    uint64_t* len = c->h_seg + c->seg_cap;
    uint64_t* pre = c->h_seg + 2 * c->seg_cap;
    uint64_t acc = 0;
    for (size_t i = 0; i < m; ++i) {
        off[i] = v[i].first;
        len[i] = v[i].second;
        pre[i] = acc;
        acc += (v[i].second + tile - 1) / tile;
    }
    pre[m] = acc;
    if ((st = grow_tile_scratch(c, acc))) return st;
    uint64_t* tb = c->h_tb;
    for (size_t i = 0; i < m; ++i) {
        const uint64_t e = off[i] + len[i];
        for (uint64_t b = off[i]; b < e; b += tile, tb += 2) {
            tb[0] = b;
            tb[1] = (e - b > tile) ? b + tile : e;
        }
    }
    *nseg_out = (int)m;
    *ntiles_out = acc;
    return BSG_OK;
}

std::mutex g_default_mu;
bsg_ctx* g_default = nullptr;

}  // namespace

// =================================================================== C ABI
extern "C" {

const char* bsg_strerror(int status) {
    switch (status) {
        case BSG_OK: return "ok";
        case BSG_ERR_INVALID_ARG: return "invalid argument";
        case BSG_ERR_NO_DEVICE: return "no usable sm_103 CUDA device";
        case BSG_ERR_CUDA: return "CUDA runtime error";
        case BSG_ERR_OUT_OF_MEMORY: return "out of memory";
        case BSG_ERR_CAPACITY: return "more options than the context capacity";
        case BSG_ERR_MISALIGNED: return "misaligned pointer";
        case BSG_ERR_TIMEOUT: return "timed out";
        case BSG_ERR_BUDGET: return "request exceeds the admission budget";
        case BSG_ERR_CANCELLED: return "cancelled";
        case BSG_ERR_NOT_SUPPORTED: return "not supported";
        case BSG_ERR_STATE: return "invalid state";
        default: return "unknown status";
    }
}

const char* bsg_last_error(const bsg_ctx* ctx) {
    return ctx ? ctx->err.c_str() : "";
}

int bsg_create(bsg_ctx** out, int device, size_t max_options) {
    if (!out) return BSG_ERR_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        return BSG_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= ndev) return BSG_ERR_NO_DEVICE;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return BSG_ERR_NO_DEVICE;
    if (!(prop.major == 10 && prop.minor == 3)) return BSG_ERR_NO_DEVICE;  // sm_103a cubin only
    if (max_options > ((size_t)1 << 36)) return BSG_ERR_INVALID_ARG;

    bsg_ctx* c = new (std::nothrow) bsg_ctx();
    if (!c) return BSG_ERR_OUT_OF_MEMORY;
    c->device = device;
    c->sm_count = prop.multiProcessorCount;
    int rc = BSG_OK;
    do {
        if (cudaSetDevice(device) != cudaSuccess) { rc = BSG_ERR_NO_DEVICE; break; }
        if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) { rc = BSG_ERR_CUDA; break; }
        if (cudaEventCreateWithFlags(&c->seg_ev, cudaEventDisableTiming) != cudaSuccess) { rc = BSG_ERR_CUDA; break; }
        c->cap = max_options;
        c->debug = debug_env();
        // 256-byte aligned arrays, each followed by guard words in debug mode
        c->cap_al = round_up(std::max<size_t>(max_options, 1) + (c->debug ? kGuardWords : 0), 64);
        if (cudaMalloc(&c->dev_buf, 7 * c->cap_al * sizeof(float)) != cudaSuccess) { rc = BSG_ERR_OUT_OF_MEMORY; break; }
        if (c->debug) {
            if (cudaMalloc(&c->d_guard, 16) != cudaSuccess) { rc = BSG_ERR_OUT_OF_MEMORY; break; }
            if (cudaMemsetAsync(c->dev_buf, kGuardByte, 7 * c->cap_al * sizeof(float), c->stream) != cudaSuccess) { rc = BSG_ERR_CUDA; break; }
        }
        c->cursor_cap = 128;
        if (cudaMalloc(&c->d_cursor, c->cursor_cap * 8) != cudaSuccess) { rc = BSG_ERR_OUT_OF_MEMORY; break; }
        if (cudaMalloc(&c->d_acc, sizeof(bsg::ErrAcc) * bsg::kMaxErrBuckets) != cudaSuccess) { rc = BSG_ERR_OUT_OF_MEMORY; break; }
        if (cudaMalloc(&c->d_edges, sizeof(double) * (bsg::kMaxErrBuckets + 1)) != cudaSuccess) { rc = BSG_ERR_OUT_OF_MEMORY; break; }
        const int bps = bsg::batch_blocks_per_sm();
        if (bps > 0) c->batch_blocks_per_sm = bps;
    } while (0);
    if (rc != BSG_OK) {
        cudaGetLastError();
        bsg_destroy(c);
        return rc;
    }
    *out = c;
    return BSG_OK;
}

void bsg_destroy(bsg_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->copy_in) cudaStreamSynchronize(c->copy_in);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->copy_out) cudaStreamSynchronize(c->copy_out);
    for (int b = 0; b < 2; ++b) {
        if (c->ev_in[b]) cudaEventDestroy(c->ev_in[b]);
        if (c->ev_comp[b]) cudaEventDestroy(c->ev_comp[b]);
        if (c->ev_out[b]) cudaEventDestroy(c->ev_out[b]);
    }
    if (c->copy_in) cudaStreamDestroy(c->copy_in);
    if (c->copy_out) cudaStreamDestroy(c->copy_out);
    if (c->dev_buf2) cudaFree(c->dev_buf2);
    graph_drop_all(c);
    if (c->dev_buf) cudaFree(c->dev_buf);
    if (c->d_seg) cudaFree(c->d_seg);
    if (c->h_seg) cudaFreeHost(c->h_seg);
    if (c->d_tb) cudaFree(c->d_tb);
    if (c->h_tb) cudaFreeHost(c->h_tb);
    if (c->d_cursor) cudaFree(c->d_cursor);
    if (c->d_acc) cudaFree(c->d_acc);
    if (c->d_edges) cudaFree(c->d_edges);
    if (c->d_guard) cudaFree(c->d_guard);
    if (c->d_sw) cudaFree(c->d_sw);
    if (c->seg_ev) cudaEventDestroy(c->seg_ev);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

void* bsg_stream(bsg_ctx* c) { return c ? (void*)c->stream : nullptr; }

int bsg_synchronize(bsg_ctx* c) {
    if (!c) return BSG_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(c->mu);
    BSG_CK(c, cudaSetDevice(c->device));
    int st = drain_pipeline(c);
    if (st) return st;
    BSG_CK(c, cudaStreamSynchronize(c->stream));
    if ((st = check_bulk_error(c))) return st;
    return debug_check(c, c->cap);
}

uint64_t bsg_kernel_launches(const bsg_ctx* c) { return c ? c->launches : 0; }

void* bsg_host_alloc(size_t bytes) {
    void* p = nullptr;
    if (cudaMallocHost(&p, bytes ? bytes : 1) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}

void bsg_host_free(void* p) {
    if (p) cudaFreeHost(p);
}

int bsg_price_soa(bsg_ctx* c, const float* s, const float* k, const float* r,
                  const float* v, const float* t, const int32_t* otype,
                  float* prices, size_t n, int num_runs, unsigned flags) {
    if (!c) return BSG_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(c->mu);
    bsg::NvtxRange nvtx_("bsg_price_soa");
    try {
        const int mode = mode_of(flags);
        if (mode < 0 || num_runs < 0) return fail(c, BSG_ERR_INVALID_ARG, "bad mode flag or num_runs");
        if (n > ((size_t)1 << 36)) return fail(c, BSG_ERR_INVALID_ARG, "n too large");
        if (n == 0 || num_runs == 0) return BSG_OK;
        BSG_CK(c, cudaSetDevice(c->device));
        bsg::SoA a{s, k, r, v, t, otype, prices};
        int st;
        if (flags & BSG_DEVICE_PTRS) {
            if ((st = check_soa_dev(c, a, n, 4))) return st;
            if ((st = enqueue_map_runs(c, a, (int64_t)n, num_runs, mode, flags))) return st;
            return finish(c, flags);
        }
        if ((st = check_soa_host(c, a))) return st;
        if (n > c->cap) return fail(c, BSG_ERR_CAPACITY, "n exceeds the context's max_options");
        if (flags & BSG_ASYNC) return enqueue_host_pipelined(c, a, n, num_runs, mode, flags);
        if ((st = drain_pipeline(c))) return st;
        if ((st = debug_arm(c, n))) return st;
        const bsg::SoA d = c->resident(n);
        const size_t b = n * 4;
        BSG_CK(c, cudaMemcpyAsync((void*)d.s, s, b, cudaMemcpyHostToDevice, c->stream));
        BSG_CK(c, cudaMemcpyAsync((void*)d.k, k, b, cudaMemcpyHostToDevice, c->stream));
        BSG_CK(c, cudaMemcpyAsync((void*)d.r, r, b, cudaMemcpyHostToDevice, c->stream));
        BSG_CK(c, cudaMemcpyAsync((void*)d.v, v, b, cudaMemcpyHostToDevice, c->stream));
        BSG_CK(c, cudaMemcpyAsync((void*)d.t, t, b, cudaMemcpyHostToDevice, c->stream));
        BSG_CK(c, cudaMemcpyAsync((void*)d.ot, otype, b, cudaMemcpyHostToDevice, c->stream));
        if ((st = enqueue_map_runs(c, d, (int64_t)n, num_runs, mode, flags))) return st;
        BSG_CK(c, cudaMemcpyAsync(prices, d.out, b, cudaMemcpyDeviceToHost, c->stream));
        BSG_CK(c, cudaStreamSynchronize(c->stream));
        if ((st = check_bulk_error(c))) return st;
        return debug_check(c, n);
    } catch (const std::bad_alloc&) {
        return fail(c, BSG_ERR_OUT_OF_MEMORY, "host allocation failed");
    }
}

int bsg_BlkSchlsEqEuroNoDiv(float* OptionPrice, int numOptions, float* sptprice,
                            float* strike, float* rate, float* volatility,
                            float* time, int* otype, float timet) {
    (void)timet;  // unused by the reference too
    if (numOptions < 0) return BSG_ERR_INVALID_ARG;
    if (numOptions == 0) return BSG_OK;
    std::lock_guard<std::mutex> lk(g_default_mu);
    if (!g_default || g_default->cap < (size_t)numOptions) {
        if (g_default) bsg_destroy(g_default);
        g_default = nullptr;
        size_t cap = std::max<size_t>((size_t)numOptions, (size_t)1 << 16);
        int st = bsg_create(&g_default, 0, cap);
        if (st) return st;
    }
    return bsg_price_soa(g_default, sptprice, strike, rate, volatility, time,
                         (const int32_t*)otype, OptionPrice, (size_t)numOptions, 1,
                         BSG_HOST_PTRS);
}

int bsg_price_fp64(bsg_ctx* c, const float* s, const float* k, const float* r,
                   const float* v, const float* t, const int32_t* otype,
                   double* out, size_t n, unsigned flags) {
    if (!c) return BSG_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(c->mu);
    if (n == 0) return BSG_OK;
    if (n > ((size_t)1 << 36)) return fail(c, BSG_ERR_INVALID_ARG, "n too large");
    BSG_CK(c, cudaSetDevice(c->device));
    bsg::SoA a{s, k, r, v, t, otype, nullptr};
    int st;
    if (flags & BSG_DEVICE_PTRS) {
        if ((st = check_soa_dev(c, a, n, 0))) return st;
        if ((st = check_dev_range(c, out, n * 8, "out"))) return st;
        cudaError_t e = bsg::launch_fp64(a, out, (int64_t)n, c->sm_count, c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "launch_fp64");
        c->launches++;
        return finish(c, flags);
    }
    if (!s || !k || !r || !v || !t || !otype || !out)
        return fail(c, BSG_ERR_INVALID_ARG, "a host array is NULL");
    if (n > c->cap) return fail(c, BSG_ERR_CAPACITY, "n exceeds the context's max_options");
    // the resident set may still be in use by pipelined calls
    if ((st = drain_pipeline(c))) return st;
    const bsg::SoA d = c->resident(n);
    const size_t b = n * 4;
    double* dout = nullptr;
    BSG_CK(c, cudaMalloc(&dout, n * 8));
    std::unique_ptr<double, decltype(&cudaFree)> guard(dout, &cudaFree);
    BSG_CK(c, cudaMemcpyAsync((void*)d.s, s, b, cudaMemcpyHostToDevice, c->stream));
    BSG_CK(c, cudaMemcpyAsync((void*)d.k, k, b, cudaMemcpyHostToDevice, c->stream));
    BSG_CK(c, cudaMemcpyAsync((void*)d.r, r, b, cudaMemcpyHostToDevice, c->stream));
    BSG_CK(c, cudaMemcpyAsync((void*)d.v, v, b, cudaMemcpyHostToDevice, c->stream));
    BSG_CK(c, cudaMemcpyAsync((void*)d.t, t, b, cudaMemcpyHostToDevice, c->stream));
    BSG_CK(c, cudaMemcpyAsync((void*)d.ot, otype, b, cudaMemcpyHostToDevice, c->stream));
    cudaError_t e = bsg::launch_fp64(d, dout, (int64_t)n, c->sm_count, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "launch_fp64");
    c->launches++;
    BSG_CK(c, cudaMemcpyAsync(out, dout, n * 8, cudaMemcpyDeviceToHost, c->stream));
    BSG_CK(c, cudaStreamSynchronize(c->stream));
    return debug_check(c, c->cap);
}

int bsg_price_soa_f64(bsg_ctx* c, const double* s, const double* k, const double* r,
                      const double* v, const double* t, const int32_t* otype, double* prices,
                      size_t n, int num_runs, unsigned flags) {
    if (!c) return BSG_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(c->mu);
    if (num_runs < 0 || (flags & ~(BSG_DEVICE_PTRS | BSG_ASYNC | BSG_NO_GRAPH)))
        return fail(c, BSG_ERR_INVALID_ARG, "bad flags or num_runs");
    if (n == 0 || num_runs == 0) return BSG_OK;
    if (n > ((size_t)1 << 36)) return fail(c, BSG_ERR_INVALID_ARG, "n too large");
    BSG_CK(c, cudaSetDevice(c->device));
    int st;
    if (flags & BSG_DEVICE_PTRS) {
        const size_t b = n * 8;
        if ((st = check_dev_range(c, s, b, "sptprice")) || (st = check_dev_range(c, k, b, "strike")) ||
            (st = check_dev_range(c, r, b, "rate")) || (st = check_dev_range(c, v, b, "volatility")) ||
            (st = check_dev_range(c, t, b, "otime")) || (st = check_dev_range(c, otype, n * 4, "otype")) ||
            (st = check_dev_range(c, prices, b, "prices")))
            return st;
        const bsg::SoA64 a{s, k, r, v, t, otype, prices};
        for (int j = 0; j < num_runs; ++j) {
            cudaError_t e = bsg::launch_map_f64(a, (int64_t)n, c->sm_count, c->stream);
            if (e != cudaSuccess) return cuda_fail(c, e, "launch_map_f64");
            c->launches++;
        }
        return finish(c, flags);
    }
    if (flags & BSG_ASYNC) return fail(c, BSG_ERR_INVALID_ARG, "BSG_ASYNC needs device pointers");
    if (!s || !k || !r || !v || !t || !otype || !prices)
        return fail(c, BSG_ERR_INVALID_ARG, "a host array is NULL");
    // host arrays: a temporary device copy (this mode has no resident buffers)
    const size_t al = round_up(n, 32);
    char* buf = nullptr;
    BSG_CK(c, cudaMalloc(&buf, al * (6 * 8 + 4)));
    std::unique_ptr<char, decltype(&cudaFree)> guard(buf, &cudaFree);
    double* d = reinterpret_cast<double*>(buf);
    int32_t* dot = reinterpret_cast<int32_t*>(d + 6 * al);
    const double* src[5] = {s, k, r, v, t};
    for (int j = 0; j < 5; ++j)
        BSG_CK(c, cudaMemcpyAsync(d + j * al, src[j], n * 8, cudaMemcpyHostToDevice, c->stream));
    BSG_CK(c, cudaMemcpyAsync(dot, otype, n * 4, cudaMemcpyHostToDevice, c->stream));
    const bsg::SoA64 a{d, d + al, d + 2 * al, d + 3 * al, d + 4 * al, dot, d + 5 * al};
    for (int j = 0; j < num_runs; ++j) {
        cudaError_t e = bsg::launch_map_f64(a, (int64_t)n, c->sm_count, c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "launch_map_f64");
        c->launches++;
    }
    BSG_CK(c, cudaMemcpyAsync(prices, d + 5 * al, n * 8, cudaMemcpyDeviceToHost, c->stream));
    BSG_CK(c, cudaStreamSynchronize(c->stream));
    return BSG_OK;
}

}  // extern "C"

namespace {

// bsg_price_batch without the lock (the caller holds c->mu).
int price_batch_impl(bsg_ctx* c, const float* s, const float* k, const float* r,
                     const float* v, const float* t, const int32_t* otype, float* prices,
                     size_t pool_len, const bsg_segment* segs, size_t nseg, int num_runs,
                     unsigned flags) {
    try {
        const int mode = mode_of(flags);
        if (mode < 0 || num_runs < 0) return fail(c, BSG_ERR_INVALID_ARG, "bad mode flag or num_runs");
        if (!(flags & BSG_DEVICE_PTRS)) return fail(c, BSG_ERR_NOT_SUPPORTED, "batch pools must be device memory");
        if (nseg && !segs) return fail(c, BSG_ERR_INVALID_ARG, "segs is NULL");
        if (pool_len == 0 || nseg == 0 || num_runs == 0) return BSG_OK;
        BSG_CK(c, cudaSetDevice(c->device));
        bsg::SoA a{s, k, r, v, t, otype, prices};
        int st;
        if ((st = check_soa_dev(c, a, pool_len, 4))) return st;
        if ((reinterpret_cast<uintptr_t>(s) | reinterpret_cast<uintptr_t>(k) |
             reinterpret_cast<uintptr_t>(r) | reinterpret_cast<uintptr_t>(v) |
             reinterpret_cast<uintptr_t>(t) | reinterpret_cast<uintptr_t>(otype) |
             reinterpret_cast<uintptr_t>(prices)) & 15)
            return fail(c, BSG_ERR_MISALIGNED, "batch pool arrays must be 16-byte aligned");
        const uint64_t topt = c->batch_tile;
        const int bps = (c->batch_bps > 0 && c->batch_bps < c->batch_blocks_per_sm)
                            ? c->batch_bps : c->batch_blocks_per_sm;
        const int grid = c->sm_count * bps;
        int m = 0;
        uint64_t ntiles = 0;
        if ((st = build_segments(c, segs, nseg, pool_len, topt, &m, &ntiles))) return st;
        if (m == 0) return finish(c, flags);
        const uint64_t* d_off = c->d_seg;
        const uint64_t* d_len = c->d_seg + c->seg_cap;
        const uint64_t* d_pre = c->d_seg + 2 * c->seg_cap;
        // table upload (3 copies of the used prefix of each array)
        BSG_CK(c, cudaMemcpyAsync((void*)d_off, c->h_seg, m * 8, cudaMemcpyHostToDevice, c->stream));
        BSG_CK(c, cudaMemcpyAsync((void*)d_len, c->h_seg + c->seg_cap, m * 8, cudaMemcpyHostToDevice, c->stream));
        BSG_CK(c, cudaMemcpyAsync((void*)d_pre, c->h_seg + 2 * c->seg_cap, (m + 1) * 8, cudaMemcpyHostToDevice, c->stream));
        BSG_CK(c, cudaMemcpyAsync(c->d_tb, c->h_tb, ntiles * 16, cudaMemcpyHostToDevice, c->stream));
        BSG_CK(c, cudaEventRecord(c->seg_ev, c->stream));
        // one work counter per pass, zeroed together, so that pass j + 1 can
        // start (PDL) while pass j drains
        if ((size_t)num_runs > c->cursor_cap) {
            BSG_CK(c, cudaStreamSynchronize(c->stream));
            graph_drop_all(c);
            cudaFree(c->d_cursor);
            c->d_cursor = nullptr;
            c->cursor_cap = 0;
            BSG_CK(c, cudaMalloc(&c->d_cursor, (size_t)num_runs * 8));
            c->cursor_cap = (size_t)num_runs;
        }
        auto all_runs = [&]() -> cudaError_t {
            cudaError_t e = cudaMemsetAsync(c->d_cursor, 0, (size_t)num_runs * 8, c->stream);
            for (int j = 0; j < num_runs && e == cudaSuccess; ++j)
                e = bsg::launch_batch(a, d_off, d_len, d_pre, c->d_tb, m, ntiles, topt,
                                      c->d_cursor + j, mode, grid, j > 0 ? 1 : 0, c->stream);
            return e;
        };
        if (num_runs == 1 || (flags & BSG_NO_GRAPH)) {
            cudaError_t e = all_runs();
            if (e != cudaSuccess) return cuda_fail(c, e, "launch_batch");
            c->launches += (uint64_t)num_runs;
            return finish(c, flags);
        }
        GraphKey key = make_key(a, (int64_t)pool_len, num_runs, mode, c->tune, 1, ntiles, m,
                                topt, grid);
        cudaGraphExec_t exec = graph_find(c, key);
        if (!exec) {
            cudaGraph_t g = nullptr;
            BSG_CK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            cudaError_t le = all_runs();
            cudaError_t ce = cudaStreamEndCapture(c->stream, &g);
            if (le != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                return cuda_fail(c, le, "launch_batch (capture)");
            }
            if (ce != cudaSuccess) return cuda_fail(c, ce, "cudaStreamEndCapture");
            cudaError_t ie = cudaGraphInstantiate(&exec, g, 0);
            cudaGraphDestroy(g);
            if (ie != cudaSuccess) return cuda_fail(c, ie, "cudaGraphInstantiate");
            graph_put(c, key, exec);
        }
        BSG_CK(c, cudaGraphLaunch(exec, c->stream));
        c->launches += (uint64_t)num_runs;
        return finish(c, flags);
    } catch (const std::bad_alloc&) {
        return fail(c, BSG_ERR_OUT_OF_MEMORY, "host allocation failed");
    }
}

}  // namespace

extern "C" {

int bsg_price_batch(bsg_ctx* c, const float* s, const float* k, const float* r,
                    const float* v, const float* t, const int32_t* otype,
                    float* prices, size_t pool_len, const bsg_segment* segs,
                    size_t nseg, int num_runs, unsigned flags) {
    if (!c) return BSG_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(c->mu);
    bsg::NvtxRange nvtx_("bsg_price_batch");
    return price_batch_impl(c, s, k, r, v, t, otype, prices, pool_len, segs, nseg, num_runs, flags);
}

int bsg_autotune_batch(bsg_ctx* c, const float* s, const float* k, const float* r,
                       const float* v, const float* t, const int32_t* otype, float* prices,
                       size_t pool_len, const bsg_segment* segs, size_t nseg,
                       bsg_batch_tune* out) {
    if (!c) return BSG_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(c->mu);
    BSG_CK(c, cudaSetDevice(c->device));
    cudaEvent_t e0, e1;
    BSG_CK(c, cudaEventCreate(&e0));
    BSG_CK(c, cudaEventCreate(&e1));
    const uint64_t keep_tile = c->batch_tile;
    const int keep_bps = c->batch_bps;
    float best_ms = 1e30f;
    bsg_batch_tune best{keep_tile, keep_bps};
    int st = BSG_OK;
    for (uint64_t tile : {2048ull, 4096ull, 8192ull, 16384ull, 32768ull}) {
        for (int bps = 1; bps <= c->batch_blocks_per_sm && st == BSG_OK; ++bps) {
            c->batch_tile = tile;
            c->batch_bps = bps;
            const unsigned f = BSG_DEVICE_PTRS | BSG_ASYNC;
            st = price_batch_impl(c, s, k, r, v, t, otype, prices, pool_len, segs, nseg, 1, f);
            if (st) break;
            cudaEventRecord(e0, c->stream);
            for (int i = 0; i < 3 && st == BSG_OK; ++i)
                st = price_batch_impl(c, s, k, r, v, t, otype, prices, pool_len, segs, nseg, 1, f);
            cudaEventRecord(e1, c->stream);
            if (st) break;
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best_ms) {
                best_ms = ms;
                best = bsg_batch_tune{tile, bps};
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) {
        c->batch_tile = keep_tile;
        c->batch_bps = keep_bps;
        return st;
    }
    BSG_CK(c, cudaStreamSynchronize(c->stream));
    c->batch_tile = best.tile_options;
    c->batch_bps = best.blocks_per_sm;
    if (out) *out = best;
    return BSG_OK;
}

int bsg_get_batch_tune(const bsg_ctx* c, bsg_batch_tune* out) {
    if (!c || !out) return BSG_ERR_INVALID_ARG;
    out->tile_options = c->batch_tile;
    out->blocks_per_sm = c->batch_bps;
    return BSG_OK;
}

int bsg_set_batch_tune(bsg_ctx* c, const bsg_batch_tune* t) {
    if (!c || !t || t->tile_options < 256 || t->tile_options > (1ull << 24) ||
        t->blocks_per_sm < 0 || t->blocks_per_sm > 64)
        return BSG_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(c->mu);
    c->batch_tile = t->tile_options;
    c->batch_bps = t->blocks_per_sm;
    return BSG_OK;
}

int bsg_price_books_plain(bsg_ctx* c, const float* s, const float* k, const float* r,
                          const float* v, const float* t, const int32_t* otype,
                          float* prices, size_t pool_len, const bsg_segment* segs,
                          size_t nseg, int num_runs, unsigned flags) {
    if (!c) return BSG_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(c->mu);
    const int mode = mode_of(flags);
    if (mode < 0 || num_runs < 0) return fail(c, BSG_ERR_INVALID_ARG, "bad mode flag or num_runs");
    if (!(flags & BSG_DEVICE_PTRS)) return fail(c, BSG_ERR_NOT_SUPPORTED, "batch pools must be device memory");
    if (nseg && !segs) return fail(c, BSG_ERR_INVALID_ARG, "segs is NULL");
    if (pool_len == 0 || nseg == 0 || num_runs == 0) return BSG_OK;
    BSG_CK(c, cudaSetDevice(c->device));
    bsg::SoA a{s, k, r, v, t, otype, prices};
    int st;
    if ((st = check_soa_dev(c, a, pool_len, 4))) return st;
    for (size_t i = 0; i < nseg; ++i) {
        const uint64_t o = segs[i].offset, l = segs[i].len;
        if (o > pool_len || l > pool_len - o)
            return fail(c, BSG_ERR_INVALID_ARG, "segment " + std::to_string(i) + " lies outside the pool");
    }
    for (int j = 0; j < num_runs; ++j) {
        for (size_t i = 0; i < nseg; ++i) {
            if (!segs[i].len) continue;
            const uint64_t o = segs[i].offset;
            bsg::SoA b{s + o, k + o, r + o, v + o, t + o, otype + o, prices + o};
            cudaError_t e = bsg::launch_map(b, (int64_t)segs[i].len, mode,
                                            bsg::pass_cfg(c->tune, j, num_runs), c->sm_count,
                                            c->stream);
            if (e != cudaSuccess) return cuda_fail(c, e, "launch_map (per book)");
            c->launches++;
        }
    }
    return finish(c, flags);
}

int bsg_error_report(bsg_ctx* c, const float* s, const float* k, const float* r,
                     const float* v, const float* t, const int32_t* otype,
                     const float* prices, size_t n, const double* edges,
                     int nbuckets, double rel_floor, bsg_err_bucket* out) {
    if (!c) return BSG_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(c->mu);
    if (!edges || !out || nbuckets < 1 || nbuckets > BSG_MAX_ERR_BUCKETS)
        return fail(c, BSG_ERR_INVALID_ARG, "bad bucket arguments");
    for (int i = 0; i < nbuckets; ++i)
        if (!(edges[i] < edges[i + 1])) return fail(c, BSG_ERR_INVALID_ARG, "bucket edges must ascend");
    BSG_CK(c, cudaSetDevice(c->device));
    bsg::SoA a{s, k, r, v, t, otype, nullptr};
    int st;
    if (n) {
        if ((st = check_soa_dev(c, a, n, 0))) return st;
        if ((st = check_dev_range(c, prices, n * 4, "prices"))) return st;
    }
    BSG_CK(c, cudaMemsetAsync(c->d_acc, 0, sizeof(bsg::ErrAcc) * nbuckets, c->stream));
    BSG_CK(c, cudaMemcpyAsync(c->d_edges, edges, sizeof(double) * (nbuckets + 1), cudaMemcpyHostToDevice, c->stream));
    if (n) {
        cudaError_t e = bsg::launch_err_report(a, prices, (int64_t)n, c->d_edges, nbuckets,
                                               rel_floor, c->d_acc, c->sm_count, c->stream);
        if (e != cudaSuccess) return cuda_fail(c, e, "launch_err_report");
        c->launches++;
    }
    std::vector<bsg::ErrAcc> h(nbuckets);
    BSG_CK(c, cudaMemcpyAsync(h.data(), c->d_acc, sizeof(bsg::ErrAcc) * nbuckets, cudaMemcpyDeviceToHost, c->stream));
    BSG_CK(c, cudaStreamSynchronize(c->stream));
    for (int i = 0; i < nbuckets; ++i) {
        out[i].count = h[i].count;
        long long b;
        std::memcpy(&b, &h[i].max_abs_bits, 8); std::memcpy(&out[i].max_abs, &b, 8);
        std::memcpy(&b, &h[i].max_rel_bits, 8); std::memcpy(&out[i].max_rel, &b, 8);
        std::memcpy(&b, &h[i].max_price_bits, 8); std::memcpy(&out[i].max_price, &b, 8);
        out[i].sum_sq_abs = h[i].sum_sq;
    }
    return BSG_OK;
}

int bsg_selftest_wait_timeout(bsg_ctx* c, double limit_s, double* elapsed_s) {
    if (!c || !(limit_s > 0) || limit_s > 10.0) return BSG_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(c->mu);
    BSG_CK(c, cudaSetDevice(c->device));
    const size_t n = 4096;  // one tile of the <4, 4> ring per CTA that runs
    if (n > c->cap) return fail(c, BSG_ERR_CAPACITY, "context too small for the self-test");
    int st = drain_pipeline(c);
    if (st) return st;
    bsg::bulk_error_take();
    const bsg::SoA d = c->resident(n);
    cudaError_t e = bsg::launch_fill(d, (int64_t)n, 7u, c->sm_count, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "launch_fill");
    const auto t0 = std::chrono::steady_clock::now();
    e = bsg::launch_bulk_wait_selftest(d, (int64_t)n, c->sm_count, (uint64_t)(limit_s * 1e9),
                                       c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "launch_bulk_wait_selftest");
    c->launches += 2;
    BSG_CK(c, cudaStreamSynchronize(c->stream));
    if (elapsed_s)
        *elapsed_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (bsg::bulk_error_take())
        return fail(c, BSG_ERR_TIMEOUT, "the staged kernel's bounded wait expired (self-test)");
    return BSG_OK;
}

int bsg_selftest_guard(bsg_ctx* c) {
    if (!c) return BSG_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(c->mu);
    if (!c->debug) return fail(c, BSG_ERR_NOT_SUPPORTED, "the context was created without BSG_DEBUG");
    BSG_CK(c, cudaSetDevice(c->device));
    int st = drain_pipeline(c);
    if (st) return st;
    // the last word of set 0's price array: a guard word (cap_al >= cap + 64)
    uint32_t* w = reinterpret_cast<uint32_t*>(c->dev_buf) + 7 * c->cap_al - 1;
    BSG_CK(c, cudaMemsetAsync(w, 0x5A, 4, c->stream));
    st = debug_check(c, c->cap);
    BSG_CK(c, cudaMemsetAsync(w, kGuardByte, 4, c->stream));
    BSG_CK(c, cudaStreamSynchronize(c->stream));
    return st;
}

int bsg_get_tune(const bsg_ctx* c, bsg_tune* out) {
    if (!c || !out) return BSG_ERR_INVALID_ARG;
    out->vec_per_thread = c->tune.vpt;
    out->block = c->tune.block;
    out->blocks_per_sm = c->tune.blocks_per_sm;
    out->load_path = c->tune.load_path;
    out->pdl = c->tune.pdl;
    out->resident_32nds = c->tune.res32;
    return BSG_OK;
}

static bool tune_valid(const bsg_tune* t) {
    const bool vpt_ok = t->vec_per_thread == 1 || t->vec_per_thread == 2 ||
                        (t->vec_per_thread == 4 && t->load_path < 2);
    const bool blk_ok = t->block == 128 || t->block == 256 || t->block == 512;
    return vpt_ok && blk_ok && t->blocks_per_sm >= 0 && t->blocks_per_sm <= 64 &&
           t->load_path >= 0 && t->load_path <= 8 && (t->pdl == 0 || t->pdl == 1) &&
           t->resident_32nds >= 0 && t->resident_32nds <= 24;
}

// The launch shape of a tuning (a resident prefix of 0 32nds means 15).
static bsg::MapCfg cfg_of(const bsg_tune& t) {
    bsg::MapCfg m{t.vec_per_thread, t.block, t.blocks_per_sm, t.load_path, t.pdl};
    m.res32 = t.resident_32nds ? t.resident_32nds : 15;
    return m;
}

int bsg_set_tune(bsg_ctx* c, const bsg_tune* t) {
    if (!c || !t) return BSG_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(c->mu);
    if (!tune_valid(t)) return fail(c, BSG_ERR_INVALID_ARG, "unsupported tuning");
    c->tune = cfg_of(*t);
    return BSG_OK;
}

}  // extern "C"

// ------------------------------------------------------------- swaptions
// The driver's per-swaption constants, rounded as the reference rounds them
// (HJM_Swaption_Blocking.cpp:48-62, 116-127), checked so that every index
// the kernel uses stays inside the path and the payment vector (the
// reference would write past its payment vector when the tenor reaches past
// the path).  Returns an empty string when the swaption is valid.
static std::string swaption_setup(const bsg_swaption& w, bsg::SwParams* p) {
    const int n = w.n_steps, nf = w.n_factors;
    if (n < 2 || n > bsg::kSwMaxSteps) return "n_steps must be 2.." + std::to_string(bsg::kSwMaxSteps);
    if (nf < 1 || nf > bsg::kSwMaxFactors)
        return "n_factors must be 1.." + std::to_string(bsg::kSwMaxFactors);
    if (!w.yield || !w.factors) return "yield or factors is NULL";
    if (!(w.years > 0) || !(w.maturity > 0) || !(w.tenor > 0) || !(w.payment_interval > 0) ||
        !(w.compounding >= 0))
        return "years, maturity, tenor and payment_interval must be > 0, compounding >= 0";
    std::memset(p, 0, sizeof(*p));
    p->h = w.years / n;
    p->sqh = std::sqrt(p->h);
    p->freq = (int)(w.payment_interval / p->h + 0.5);
    p->strike_cont = w.compounding == 0 ? w.strike
                                        : (1 / w.compounding) * std::log(1 + w.strike * w.compounding);
    p->swap_len = (int)(n - w.maturity / p->h + 0.5);
    p->start = (int)(w.maturity / p->h + 0.5);
    p->swap_points = (int)(w.tenor / p->h + 0.5);
    p->payment_interval = w.payment_interval;
    p->n_steps = n;
    p->n_factors = nf;
    p->seed = w.seed;
    if (p->freq < 1 || p->start < 1 || p->start > n - 1 || p->swap_len < 1 ||
        p->swap_len > n - p->start || p->swap_points >= p->swap_len)
        return "maturity, tenor and payment interval do not fit the grid of n_steps points over years";
    for (int i = 0; i < n; ++i) {
        p->yield[i] = w.yield[i];
        if (!std::isfinite(w.yield[i])) return "yield is not finite";
    }
    for (int k = 0; k < nf; ++k)
        for (int m = 0; m < n - 1; ++m) {
            p->vol[k][m] = w.factors[(size_t)k * (n - 1) + m];
            if (!std::isfinite(p->vol[k][m])) return "factors are not finite";
        }
    if (!std::isfinite(p->strike_cont)) return "strike is not finite";
    return std::string();
}

extern "C" int bsg_price_swaptions(bsg_ctx* c, const bsg_swaption* sw, size_t n, uint64_t trials,
                                   double* price, double* std_err) {
    if (!c) return BSG_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(c->mu);
    bsg::NvtxRange nvtx_("bsg_price_swaptions");
    if (n == 0) return BSG_OK;
    if (!sw || !price) return fail(c, BSG_ERR_INVALID_ARG, "swaptions or price is NULL");
    if (n > 65535) return fail(c, BSG_ERR_CAPACITY, "at most 65535 swaptions per call");
    if (trials < 2 || trials > ((uint64_t)1 << 40))
        return fail(c, BSG_ERR_INVALID_ARG, "trials must be 2..2^40");
    std::vector<bsg::SwParams> tab(n);
    int max_steps = 2;
    for (size_t i = 0; i < n; ++i) {
        const std::string why = swaption_setup(sw[i], &tab[i]);
        if (!why.empty()) return fail(c, BSG_ERR_INVALID_ARG, "swaption " + std::to_string(i) + ": " + why);
        max_steps = std::max(max_steps, sw[i].n_steps);
    }
    BSG_CK(c, cudaSetDevice(c->device));
    if (int st = drain_pipeline(c)) return st;
    // paths per thread: the most (up to 32; each block pays a set-up) that
    // still leave 1216 blocks, four waves of 2 blocks on 152 SMs.  A fixed
    // rule of (n, trials), so the summation order -- and the bits -- do
    // not depend on the device.
    int per_thread = 32;
    while (per_thread > 1 && n * (size_t)bsg::swaption_chunks(trials, per_thread) < 1216) per_thread /= 2;
    const size_t chunks = (size_t)bsg::swaption_chunks(trials, per_thread);
    const size_t tab_b = round_up(n * sizeof(bsg::SwParams), 256);
    const size_t part_b = round_up(2 * n * chunks * sizeof(double), 256);
    const size_t out_b = round_up(2 * n * sizeof(double), 256);
    const size_t need = tab_b + part_b + out_b;
    if (need > c->sw_cap) {
        if (c->d_sw) {
            BSG_CK(c, cudaStreamSynchronize(c->stream));
            cudaFree(c->d_sw);
            c->d_sw = nullptr;
            c->sw_cap = 0;
        }
        if (cudaMalloc(&c->d_sw, need) != cudaSuccess) {
            cudaGetLastError();
            return fail(c, BSG_ERR_OUT_OF_MEMORY, "swaption scratch");
        }
        c->sw_cap = need;
    }
    bsg::SwParams* d_tab = reinterpret_cast<bsg::SwParams*>(c->d_sw);
    double* d_part = reinterpret_cast<double*>(c->d_sw + tab_b);
    double* d_out = reinterpret_cast<double*>(c->d_sw + tab_b + part_b);
    BSG_CK(c, cudaMemcpyAsync(d_tab, tab.data(), n * sizeof(bsg::SwParams), cudaMemcpyHostToDevice,
                              c->stream));
    cudaError_t e = bsg::launch_swaptions(d_tab, (int)n, max_steps, trials, per_thread, d_part, d_out,
                                          c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "launch_swaptions");
    c->launches += 2;
    std::vector<double> out(2 * n);
    BSG_CK(c, cudaMemcpyAsync(out.data(), d_out, 2 * n * sizeof(double), cudaMemcpyDeviceToHost,
                              c->stream));
    BSG_CK(c, cudaStreamSynchronize(c->stream));
    for (size_t i = 0; i < n; ++i) {
        price[i] = out[2 * i];
        if (std_err) std_err[i] = out[2 * i + 1];
    }
    return BSG_OK;
}

extern "C" int bsg_swaption_normals(bsg_ctx* c, const uint32_t* words, size_t n_pairs, double* z) {
    if (!c) return BSG_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(c->mu);
    if (n_pairs == 0) return BSG_OK;
    if (!words || !z) return fail(c, BSG_ERR_INVALID_ARG, "words or z is NULL");
    if (n_pairs > ((size_t)1 << 26)) return fail(c, BSG_ERR_CAPACITY, "at most 2^26 pairs per call");
    BSG_CK(c, cudaSetDevice(c->device));
    if (int st = drain_pipeline(c)) return st;
    void* d = nullptr;
    const size_t wb = n_pairs * 4 * sizeof(uint32_t), zb = n_pairs * 2 * sizeof(double);
    if (cudaMalloc(&d, wb + zb) != cudaSuccess) {
        cudaGetLastError();
        return fail(c, BSG_ERR_OUT_OF_MEMORY, "swaption normals scratch");
    }
    uint32_t* dw = static_cast<uint32_t*>(d);
    double* dz = reinterpret_cast<double*>(static_cast<char*>(d) + wb);  // wb is a multiple of 16
    cudaError_t e = cudaMemcpyAsync(dw, words, wb, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = bsg::launch_swaption_normals(dw, n_pairs, dz, c->stream);
    if (e == cudaSuccess) {
        c->launches += 1;
        e = cudaMemcpyAsync(z, dz, zb, cudaMemcpyDeviceToHost, c->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(c, e, "bsg_swaption_normals");
    return BSG_OK;
}

extern "C" int bsg_HJM_Swaption_Blocking(double* pdSwaptionPrice, double dStrike,
                                         double dCompounding, double dMaturity, double dTenor,
                                         double dPaymentInterval, int iN, int iFactors,
                                         double dYears, double* pdYield, double** ppdFactors,
                                         long iRndSeed, long lTrials, int BLOCKSIZE, int tid) {
    (void)BLOCKSIZE;  // the GPU's blocking is its own
    (void)tid;
    if (!pdSwaptionPrice || !ppdFactors || iFactors < 1 || iFactors > bsg::kSwMaxFactors ||
        iN < 2 || iN > bsg::kSwMaxSteps || lTrials < 2)
        return BSG_ERR_INVALID_ARG;
    double vol[bsg::kSwMaxFactors * bsg::kSwMaxSteps];
    for (int k = 0; k < iFactors; ++k) {
        if (!ppdFactors[k]) return BSG_ERR_INVALID_ARG;
        for (int m = 0; m < iN - 1; ++m) vol[k * (iN - 1) + m] = ppdFactors[k][m];
    }
    const bsg_swaption w{dStrike, dCompounding, dMaturity, dTenor, dPaymentInterval, dYears,
                         iN, iFactors, pdYield, vol, (uint64_t)iRndSeed};
    std::lock_guard<std::mutex> lk(g_default_mu);
    if (!g_default) {
        int st = bsg_create(&g_default, 0, (size_t)1 << 16);
        if (st) return st;
    }
    const int st = bsg_price_swaptions(g_default, &w, 1, (uint64_t)lTrials, &pdSwaptionPrice[0],
                                       &pdSwaptionPrice[1]);
    return st == BSG_OK ? 1 : st;
}

// ------------------------------------------------------------- autotuner
// Times every plain-map shape on the context's device for n options and
// keeps the fastest.  The choice is cached per (device name, SM count,
// floor(log2 n)) in $BSG_TUNE_CACHE when that variable names a file.
static std::string tune_key(const bsg_ctx* c, size_t n) {
    cudaDeviceProp p;
    cudaGetDeviceProperties(&p, c->device);
    int b = 0;
    while (((size_t)1 << (b + 1)) <= n) ++b;
    std::ostringstream os;
    os << p.name << "|" << p.multiProcessorCount << "|" << b;
    return os.str();
}

// Serialises this process's reads and appends of the tuning cache file.
static std::mutex g_tune_cache_mu;

static bool tune_cache_lookup(const std::string& key, bsg_tune* t) {
    std::lock_guard<std::mutex> lk(g_tune_cache_mu);
    const char* path = std::getenv("BSG_TUNE_CACHE");
    if (!path || !*path) return false;
    std::ifstream f(path);
    std::string line;
    bool found = false;
    while (std::getline(f, line)) {
        const size_t bar = line.rfind('|');
        if (bar == std::string::npos || line.compare(0, bar, key) != 0) continue;
        bsg_tune x;
        if (std::sscanf(line.c_str() + bar + 1, "%d %d %d %d %d %d", &x.vec_per_thread, &x.block,
                        &x.blocks_per_sm, &x.load_path, &x.pdl, &x.resident_32nds) == 6 &&
            tune_valid(&x)) {
            *t = x;
            found = true;
        }
    }
    return found;
}

static void tune_cache_store(const std::string& key, const bsg_tune& t) {
    std::lock_guard<std::mutex> lk(g_tune_cache_mu);
    const char* path = std::getenv("BSG_TUNE_CACHE");
    if (!path || !*path) return;
    std::ofstream f(path, std::ios::app);
    f << key << "|" << t.vec_per_thread << " " << t.block << " " << t.blocks_per_sm << " "
      << t.load_path << " " << t.pdl << " " << t.resident_32nds << "\n";
}

extern "C" int bsg_autotune(bsg_ctx* c, size_t n, bsg_tune* out) {
    if (!c || n == 0) return BSG_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(c->mu);
    bsg::NvtxRange nvtx_("bsg_autotune");
    BSG_CK(c, cudaSetDevice(c->device));
    const std::string key = tune_key(c, n);
    bsg_tune best{};
    if (tune_cache_lookup(key, &best)) {
        c->tune = cfg_of(best);
        if (out) *out = best;
        return BSG_OK;
    }
    if (int st = drain_pipeline(c)) return st;
    // inputs: the resident buffers when they fit, else a temporary pool
    bsg::SoA a;
    char* tmp = nullptr;
    if (n <= c->cap) {
        a = c->resident(n);
    } else {
        const size_t al = round_up(n, 64);
        BSG_CK(c, cudaMalloc(&tmp, 7 * al * sizeof(float)));
        float* f = reinterpret_cast<float*>(tmp);
        a = bsg::SoA{f, f + al, f + 2 * al, f + 3 * al, f + 4 * al,
                     reinterpret_cast<const int32_t*>(f + 5 * al), f + 6 * al};
    }
    std::unique_ptr<char, decltype(&cudaFree)> guard(tmp, &cudaFree);
    cudaError_t e = bsg::launch_fill(a, (int64_t)n, 12345u, c->sm_count, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "launch_fill");
    c->launches++;
    cudaEvent_t e0, e1;
    BSG_CK(c, cudaEventCreate(&e0));
    BSG_CK(c, cudaEventCreate(&e1));
    // Times `reps` back-to-back passes (as the NUM_RUNS passes run) after one
    // warm-up pass; a negative result: the launch failed or a bounded wait of
    // the staged kernel expired (never pick such a shape).
    auto time_cfg = [&](const bsg::MapCfg& cfg, int reps) -> float {
        e = bsg::launch_map(a, (int64_t)n, bsg::MODE_FAST, cfg, c->sm_count, c->stream);
        if (e != cudaSuccess) return -1.0f;
        cudaEventRecord(e0, c->stream);
        for (int i = 0; i < reps && e == cudaSuccess; ++i)
            e = bsg::launch_map(a, (int64_t)n, bsg::MODE_FAST, bsg::pass_cfg(cfg, i, reps),
                                c->sm_count, c->stream);
        cudaEventRecord(e1, c->stream);
        c->launches += reps + 1;
        if (e != cudaSuccess) return -1.0f;
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (bsg::bulk_error_take()) return -1.0f;
        return ms;
    };
    // stage 1: every shape for 5 passes (the resident prefix at 15/32)
    std::vector<std::pair<float, bsg_tune>> timed;
    for (int lp : {0, 1, 2, 6, 7, 8})
        for (int vpt : {1, 2, 4})
            for (int block : {128, 256, 512})
                for (int bps : {0, 2, 4, 8})
                for (int pdl : {0, 1}) {
                    bsg_tune t{vpt, block, bps, lp, pdl, lp == 7 ? 15 : 0};
                    if (!tune_valid(&t) || e != cudaSuccess) continue;
                    const float ms = time_cfg(cfg_of(t), 5);
                    if (ms >= 0) timed.push_back({ms, t});
                }
    // the TMA bulk-staged kernels: three ring shapes, with and without PDL
    for (int lp : {3, 4, 5})
        for (int pdl : {0, 1}) {
            if (e != cudaSuccess) break;
            const bsg_tune t{1, 256, 0, lp, pdl, 0};
            const float ms = time_cfg(cfg_of(t), 5);
            if (ms >= 0) timed.push_back({ms, t});
        }
    std::stable_sort(timed.begin(), timed.end(),
                     [](const auto& x, const auto& y) { return x.first < y.first; });
    // stage 2: the prefix size of the fastest resident-prefix shape, over 25
    // passes (the residency only shows across many passes); every other
    // resident-prefix shape takes the size found
    int best_res = 15;
    for (const auto& x : timed) {
        if (x.second.load_path != 7) continue;
        float res_ms = 1e30f;
        for (int r32 : {4, 8, 10, 12, 14, 15, 16, 18, 20, 24}) {
            if (e != cudaSuccess) break;
            bsg_tune t = x.second;
            t.resident_32nds = r32;
            const float ms = time_cfg(cfg_of(t), 25);
            if (ms >= 0 && ms < res_ms) {
                res_ms = ms;
                best_res = r32;
            }
        }
        break;
    }
    for (auto& x : timed)
        if (x.second.load_path == 7) x.second.resident_32nds = best_res;
    // stage 3: the four fastest again over NUM_RUNS passes each (a call's
    // length: the steady state the L2 reaches across passes), three rounds
    // interleaved, the best round of each
    if (timed.size() > 4) timed.resize(4);
    std::vector<float> fin(timed.size(), 1e30f);
    for (int round = 0; round < 3 && e == cudaSuccess; ++round)
        for (size_t q = 0; q < timed.size() && e == cudaSuccess; ++q) {
            const float ms = time_cfg(cfg_of(timed[q].second), BSG_NUM_RUNS);
            if (ms >= 0 && ms < fin[q]) fin[q] = ms;
        }
    float best_ms = 1e30f;
    best = bsg_tune{1, 256, 0, 0, 0, 0};
    for (size_t q = 0; q < timed.size(); ++q)
        if (fin[q] < best_ms) {
            best_ms = fin[q];
            best = timed[q].second;
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return cuda_fail(c, e, "autotune launch");
    BSG_CK(c, cudaStreamSynchronize(c->stream));
    c->tune = cfg_of(best);
    tune_cache_store(key, best);
    if (out) *out = best;
    return BSG_OK;
}
