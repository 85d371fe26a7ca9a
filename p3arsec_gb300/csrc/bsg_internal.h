// bsg_internal.h -- launch interface between the C ABI (bsg_api.cu) and the
// kernels (bsg_kernels.cu).  Not installed; no torch types anywhere.
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

namespace bsg {

// Arithmetic of the map (see bsg_math.cuh).
enum Mode : int { MODE_FAST = 0, MODE_SFU_REF = 1, MODE_LIBM_REF = 2 };

// One SoA view: the reference's five float arrays, int32 otype, float out.
struct SoA {
    const float* s;
    const float* k;
    const float* r;
    const float* v;
    const float* t;
    const int32_t* ot;
    float* out;
};

// The FP64 product mode's SoA: double storage (otype int32).
struct SoA64 {
    const double* s;
    const double* k;
    const double* r;
    const double* v;
    const double* t;
    const int32_t* ot;
    double* out;
};

// Plain-map launch shape (see bsg_tune in bsg.h).
struct MapCfg {
    int vpt;           // vector groups per thread per tile: 1, 2, 4
    int block;         // threads per block
    int blocks_per_sm; // 0: one block per tile; else grid = blocks_per_sm * SMs
    int load_path;     // 0: v4 nc; 1: v4 + L2 evict_first; 2: v8 (256-bit) nc;
                       // 3, 4, 5: TMA bulk copies into a shared-memory ring;
                       // 6: v8 + L2 evict_first; 7: v8, a prefix of the book
                       // (res32 32nds of the L2) evict_last, the rest evict_first;
                       // 8: v8, every other pass in reverse tile order
    int pdl;           // 1: launch with programmatic stream serialization
    int res32 = 15;    // LP 7: the resident prefix, in 32nds of the L2 (1..24)
    int rev = 0;       // LP 8: this pass walks the tiles from the last to the first
};

// Accumulators of one error bucket (device scratch, zeroed per report).
struct ErrAcc {
    unsigned long long count;
    unsigned long long max_abs_bits;   // non-negative doubles order as u64
    unsigned long long max_rel_bits;
    unsigned long long max_price_bits;
    double sum_sq;
};

constexpr int kMaxErrBuckets = 32;
constexpr int kBatchBlock = 256;

// Launches one pass of the plain map over n options.  Picks the vector
// kernel when every pointer is aligned for the configured width, else the
// scalar kernel.  Returns the launch error.
cudaError_t launch_map(const SoA& a, int64_t n, int mode, const MapCfg& cfg,
                       int sm_count, cudaStream_t st);
// The shape of pass j of `runs` consecutive passes over the same book.  The
// resident-prefix load path (7) marks part of the book evict_last so that it
// stays in L2 for the next pass.  The last pass runs the same loads with
// evict_first (6): it still hits the resident lines, and an access with an
// explicit policy sets the line's priority, so no evict_last line is left
// behind the call.  A single pass therefore never marks lines evict_last.
// The alternating load path (8) walks odd passes from the book's last tile
// to its first, so each pass starts on the lines the previous pass touched
// last, which the L2 still holds.
inline MapCfg pass_cfg(MapCfg c, int j, int runs) {
    if (c.load_path == 7 && j == runs - 1) c.load_path = 6;
    c.rev = (c.load_path == 8) ? (j & 1) : 0;
    return c;
}
// Reads and clears the bulk-staged kernel's error word (non-zero: a bounded
// wait expired and some tiles were not priced).
unsigned bulk_error_take();
// Launches the bulk-staged kernel with every barrier expecting 16 bytes more
// than its copies deliver, so each wait expires after wait_ns (self-test of
// the bounded waits; the copies themselves complete normally).
cudaError_t launch_bulk_wait_selftest(const SoA& a, int64_t n, int sm_count, uint64_t wait_ns,
                                      cudaStream_t st);
// True when launch_map would take the vector path for these pointers.
bool map_vectorizable(const SoA& a, const MapCfg& cfg);

cudaError_t launch_fp64(const SoA& a, double* out, int64_t n, int sm_count,
                        cudaStream_t st);
// One pass of the FP64 product mode over n options.
cudaError_t launch_map_f64(const SoA64& a, int64_t n, int sm_count, cudaStream_t st);

// Persistent batched pricing.  seg_off/seg_len/tile_prefix are device arrays
// of nseg (tile_prefix: nseg + 1 entries, exclusive prefix of tiles of
// tile_opts options per segment); tile_bounds (optional, NULL = search the
// prefix instead) holds each tile's [begin, end) in the pool, 2 * ntiles
// entries; cursor is a device counter that must be 0 at launch.  pdl: launch
// with programmatic stream serialization (the next pass may start while
// this one drains; it must use its own cursor).
cudaError_t launch_batch(const SoA& pool, const uint64_t* seg_off,
                         const uint64_t* seg_len, const uint64_t* tile_prefix,
                         const uint64_t* tile_bounds, int nseg, uint64_t ntiles,
                         uint64_t tile_opts, unsigned long long* cursor, int mode, int grid,
                         int pdl, cudaStream_t st);
// Default options per batch tile.
uint64_t batch_tile_options();
// Resident blocks per SM of the batch kernel (its persistent grid = this x SMs).
int batch_blocks_per_sm();

cudaError_t launch_err_report(const SoA& a, const float* prices, int64_t n,
                              const double* edges, int nbuckets,
                              double rel_floor, ErrAcc* acc, int sm_count,
                              cudaStream_t st);

// NVTX range for the lifetime of a scope (header-only NVTX3: a no-op unless a
// profiler injects itself), so profiler timelines show the library's calls.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// Where [p, p + bytes) lies: kExtentOk when it is device memory of `device`
// (or managed memory) inside one allocation, or across consecutive pieces
// that the virtual memory API mapped into one range with read-write access
// for `device` (pool allocators that grow in place map memory piece by
// piece).  Ordinary allocations are never joined with their neighbours, so
// a size that runs past one is kExtentOverrun.
enum Extent : int {
    kExtentOk = 0,
    kExtentNotDevice = 1,
    kExtentOtherDevice = 2,
    kExtentUnknown = 3,
    kExtentOverrun = 4,
};
int device_extent(const void* p, size_t bytes, int device);

// ---- swaptions (HJM Monte Carlo) -------------------------------------------
constexpr int kSwMaxSteps = 32;    // grid points of the HJM path (iN)
constexpr int kSwMaxFactors = 8;   // volatility factors (iFactors)

// One swaption as the path kernel reads it: the driver's constants, already
// rounded as the reference rounds them, and the raw curves.
struct SwParams {
    double strike_cont;       // strike in continuous compounding
    double payment_interval;  // years between swap payments
    double h, sqh;            // grid step and its square root
    int n_steps, n_factors;
    int start;                // the swaption's maturity on the grid
    int swap_len;             // forward rates of the swap curve at maturity
    int freq, swap_points;    // payment every freq steps, the last at swap_points
    uint64_t seed;            // the paths' random stream
    double yield[kSwMaxSteps];
    double vol[kSwMaxFactors][kSwMaxSteps];  // [k][m], m < n_steps - 1
};

// Blocks of trials per swaption for `trials` paths, per_thread paths per thread.
int swaption_chunks(uint64_t trials, int per_thread);
// Prices nsw swaptions (device table prm) with `trials` paths each:
// out[2 i] = mean discounted payoff, out[2 i + 1] = its standard error.
// partial: device scratch of 2 * nsw * swaption_chunks(trials, per_thread)
// doubles.  max_steps: the largest n_steps in the table.
cudaError_t launch_swaptions(const SwParams* prm, int nsw, int max_steps, uint64_t trials,
                             int per_thread, double* partial, double* out, cudaStream_t st);

// z[2 i], z[2 i + 1] = the swaption kernel's normal pair of words[4 i .. 4 i + 3]
// (device arrays), i < n.
cudaError_t launch_swaption_normals(const uint32_t* words, uint64_t n, double* z, cudaStream_t st);

// Fills n options with a deterministic plausible book (autotuning input).
cudaError_t launch_fill(const SoA& a, int64_t n, uint32_t seed, int sm_count,
                        cudaStream_t st);

// Debug guards of a resident set: seven arrays of `stride` words from `base`;
// the guard of input array a < 6 is words [cap, stride), that of the price
// array words [out_lo, stride).  Adds the number of guard words that differ
// from `pattern` to res[0] and lowers res[1] to the smallest differing word's
// index from `base` (res must hold {0, ~0} beforehand).
cudaError_t launch_guard_check(const uint32_t* base, int64_t stride, int64_t cap,
                               int64_t out_lo, uint32_t pattern, unsigned long long* res,
                               int sm_count, cudaStream_t st);

}  // namespace bsg
