/*
 * bsg.h -- C ABI of libbsgpu.so, the GB300 (sm_103a) Black-Scholes map.
 *
 * Replaces the hot path of P3ARSEC's blackscholes benchmark
 * (parsec-ff/pkgs/apps/blackscholes/src/blackscholes.c): BlkSchlsEqEuroNoDiv
 * and its polynomial CNDF applied to SoA option arrays NUM_RUNS times.
 *
 * Conventions (the reference's, plus status codes):
 *  - The caller owns every buffer.  Arrays are the reference's SoA layout
 *    (blackscholes.c:103-113, 747-767): five float arrays sptprice, strike,
 *    rate, volatility, otime; int32 otype (1 = put, 0 = call); float prices.
 *  - Every call returns a bsg_status (0 = ok, < 0 = error) instead of
 *    printing and calling exit() as the reference does (blackscholes.c:697-739).
 *    bsg_last_error() gives a message for the last failure on a context.
 *  - A context owns one device, one stream, resident device buffers for up
 *    to max_options options, cached CUDA graphs and the tuning choice.  Calls
 *    on one context are serialised by a lock; use one context per host
 *    thread for concurrency.
 *  - The context's stream is non-blocking: it does not wait for work other
 *    streams have enqueued (the legacy default stream included).  Device
 *    arrays passed to a call must be complete when the call is made:
 *    synchronise their producer first, or produce them on bsg_stream()
 *    (e.g. torch.cuda.ExternalStream(bsg_stream(ctx))).  A synchronous
 *    call's results are complete when it returns; a BSG_ASYNC call's after
 *    bsg_synchronize() or in work ordered after bsg_stream().
 *  - No call ever falls back to a CPU computation: without a usable GPU,
 *    bsg_create fails with BSG_ERR_NO_DEVICE.
 */
#ifndef BSG_H
#define BSG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BSG_ABI_VERSION 2

typedef struct bsg_ctx bsg_ctx;

typedef enum bsg_status {
    BSG_OK = 0,
    BSG_ERR_INVALID_ARG = -1,   /* null pointer, negative count, bad flag */
    BSG_ERR_NO_DEVICE = -2,     /* no CUDA device / bad ordinal / not sm_103 */
    BSG_ERR_CUDA = -3,          /* a CUDA runtime call failed */
    BSG_ERR_OUT_OF_MEMORY = -4, /* device or pinned host allocation failed */
    BSG_ERR_CAPACITY = -5,      /* n exceeds the context's max_options */
    BSG_ERR_MISALIGNED = -6,    /* device pointer not 4-byte aligned */
    BSG_ERR_TIMEOUT = -7,       /* a bounded wait expired */
    BSG_ERR_BUDGET = -8,        /* request larger than the admission budget */
    BSG_ERR_CANCELLED = -9,     /* request cancelled while queued */
    BSG_ERR_NOT_SUPPORTED = -10,
    BSG_ERR_STATE = -11         /* call not valid in the object's state */
} bsg_status;

/* ---- flags ------------------------------------------------------------ */
#define BSG_HOST_PTRS     0x000u /* host arrays: copied in and out inside the call */
#define BSG_DEVICE_PTRS   0x001u /* device arrays on the context's device */
#define BSG_ASYNC         0x002u /* return once enqueued (see bsg_price_soa) */
#define BSG_MODE_FAST     0x000u /* compensated FP32 with SFU approximations */
#define BSG_MODE_SFU_REF  0x010u /* reference operation order, SFU approximations */
#define BSG_MODE_LIBM_REF 0x020u /* reference operation order, correctly rounded exp/log,
                                    IEEE division and square root: the reference's own
                                    FP32 prices wherever glibc's expf/logf round correctly
                                    (99.7 % of options); compute-bound, ~3x slower */
#define BSG_MODE_MASK     0x0F0u
#define BSG_NO_GRAPH      0x100u /* launch NUM_RUNS kernels directly, no graph */

#define BSG_NUM_RUNS 100 /* blackscholes.c:87 */

/* ---- context ---------------------------------------------------------- */

/* New context on CUDA device `device` able to price up to max_options per
 * call with host pointers (device-pointer calls have no size limit).
 * Allocates 28 * max_options bytes of device memory.
 * Debug guards: with the environment variable BSG_DEBUG set (and not "0")
 * when the context is created, every resident array is followed by at least
 * 64 guard words; each synchronous call then checks that no kernel or copy
 * wrote past the options it was given (the resident prices past n included)
 * and returns BSG_ERR_STATE, naming the first overwritten word, if one did.
 * Off by default: the check costs a launch and a synchronisation per call. */
int bsg_create(bsg_ctx** out, int device, size_t max_options);
void bsg_destroy(bsg_ctx* ctx);
const char* bsg_strerror(int status);
const char* bsg_last_error(const bsg_ctx* ctx);
/* The context's cudaStream_t (as void*): work of every call is ordered on it. */
void* bsg_stream(bsg_ctx* ctx);
/* Waits for every call enqueued on the context (pipelined host calls too). */
int bsg_synchronize(bsg_ctx* ctx);
/* Number of kernels this context has launched so far. */
uint64_t bsg_kernel_launches(const bsg_ctx* ctx);

/* Pinned host memory for staging (cudaMallocHost); NULL on failure. */
void* bsg_host_alloc(size_t bytes);
void bsg_host_free(void* p);

/* ---- the map -----------------------------------------------------------
 * prices[i] = BlkSchlsEqEuroNoDiv(sptprice[i], strike[i], rate[i],
 *             volatility[i], otime[i], otype[i]) for i < n, evaluated
 * num_runs times (each run a full pass over the n options, as the
 * reference's NUM_RUNS loop, blackscholes.c:315-348 / 607-658).
 * Replaces bs_thread (blackscholes.c:607) and the FastFlow map's svc
 * (blackscholes.c:316-346).  n == 0 or num_runs == 0 is a no-op.
 * BSG_ASYNC with device pointers: returns once enqueued on bsg_stream().
 * BSG_ASYNC with host pointers (pipelined): returns once enqueued; successive
 * calls alternate between two resident buffer sets and overlap one call's
 * host<->device copies with another's passes.  The caller keeps the host
 * arrays (pinned, for real overlap) unchanged until bsg_synchronize. */
int bsg_price_soa(bsg_ctx* ctx, const float* sptprice, const float* strike,
                  const float* rate, const float* volatility,
                  const float* otime, const int32_t* otype, float* prices,
                  size_t n, int num_runs, unsigned flags);

/* The reference's batch signature (blackscholes.simd.c:221-223): one pass
 * over numOptions options on the default context of device 0, host
 * pointers.  timet is unused, as in the reference. */
int bsg_BlkSchlsEqEuroNoDiv(float* OptionPrice, int numOptions, float* sptprice,
                            float* strike, float* rate, float* volatility,
                            float* time, int* otype, float timet);

/* FP64 product mode: double storage in and out, the types of the
 * reference's SIMD variant built with NCO = 2 (blackscholes.simd.c:68-81,
 * 221-298), num_runs passes.  Bound by the GPU's FP64 rate.  Host or device
 * pointers as bsg_price_soa (host calls stage through temporary device
 * memory). */
int bsg_price_soa_f64(bsg_ctx* ctx, const double* sptprice, const double* strike,
                      const double* rate, const double* volatility,
                      const double* otime, const int32_t* otype, double* prices,
                      size_t n, int num_runs, unsigned flags);

/* FP64 evaluation of the same formula (validation oracle kernel).  Same
 * pointer rules as bsg_price_soa; out is double. */
int bsg_price_fp64(bsg_ctx* ctx, const float* sptprice, const float* strike,
                   const float* rate, const float* volatility,
                   const float* otime, const int32_t* otype, double* out,
                   size_t n, unsigned flags);

/* ---- batched books -----------------------------------------------------
 * Many independent books stored in one SoA pool of pool_len options; book b
 * occupies [segs[b].offset, segs[b].offset + segs[b].len).  One persistent
 * kernel prices every book (tiles handed out by a device work counter), and
 * num_runs passes are replayed from a captured CUDA graph.  Pool pointers
 * are device pointers; segs is a host array.  Segments must lie inside the
 * pool; they may be in any order but must not overlap. */
typedef struct bsg_segment {
    uint64_t offset;
    uint64_t len;
} bsg_segment;

int bsg_price_batch(bsg_ctx* ctx, const float* sptprice, const float* strike,
                    const float* rate, const float* volatility,
                    const float* otime, const int32_t* otype, float* prices,
                    size_t pool_len, const bsg_segment* segs, size_t nseg,
                    int num_runs, unsigned flags);

/* Shape of the persistent batch kernel: options per tile handed out by the
 * work counter, and resident blocks per SM (0 = as many as fit). */
typedef struct bsg_batch_tune {
    uint64_t tile_options;
    int blocks_per_sm;
} bsg_batch_tune;

/* Times the batch kernel's shapes (tile 2048..32768 options x 1..max blocks
 * per SM) on these books (one pass each, prices written) and makes the
 * fastest the context's choice. */
int bsg_autotune_batch(bsg_ctx* ctx, const float* sptprice, const float* strike,
                       const float* rate, const float* volatility,
                       const float* otime, const int32_t* otype, float* prices,
                       size_t pool_len, const bsg_segment* segs, size_t nseg,
                       bsg_batch_tune* out);
int bsg_get_batch_tune(const bsg_ctx* ctx, bsg_batch_tune* out);
int bsg_set_batch_tune(bsg_ctx* ctx, const bsg_batch_tune* tune);

/* The same books priced by one plain map launch per book (the comparison
 * baseline for bsg_price_batch). */
int bsg_price_books_plain(bsg_ctx* ctx, const float* sptprice, const float* strike,
                          const float* rate, const float* volatility,
                          const float* otime, const int32_t* otype, float* prices,
                          size_t pool_len, const bsg_segment* segs, size_t nseg,
                          int num_runs, unsigned flags);

/* ---- batched books without allocation ----------------------------------
 * No counterpart in the reference.  For callers that may not allocate
 * memory (code under a fixed device-memory budget or inside another
 * runtime's allocator, plugins that must not allocate after start-up,
 * real-time loops where an allocation can block): the same pricing as
 * bsg_price_batch with no context and no allocation of any kind.  Its
 * scratch (segment table, tile prefix, tile counter; 164,104 bytes) is a
 * fixed device array that every GPU loading this library holds until exit.
 *  - Runs on the calling thread's current device, on `stream` (a
 *    cudaStream_t, NULL = legacy default stream).  Pool arrays are device
 *    memory, 16-byte aligned; segs is a host array.  flags: BSG_DEVICE_PTRS
 *    is implied; BSG_ASYNC returns once enqueued (keep segs alive until the
 *    stream reaches the call when it is pinned memory).  It prices in the
 *    fast mode only: any other flag, BSG_MODE_SFU_REF and BSG_MODE_LIBM_REF
 *    included, is BSG_ERR_INVALID_ARG (checked before any CUDA call).
 *  - The first call on a device looks up the scratch array's device address
 *    (cudaGetSymbolAddress); make that first call before any stream capture.
 *    The address is kept per device together with the driver context it was
 *    found in; after a device reset (a new primary context) the next call
 *    looks it up again.
 *  - nseg above BSG_NOALLOC_MAX_SEGMENTS returns BSG_ERR_CAPACITY.
 *  - Every call reuses the same scratch: calls that overlap on the GPU race
 *    and give wrong prices (never writes outside their own pool).  Serialise
 *    them on one stream.  Overlapping segments are priced twice (same values).
 */
#define BSG_NOALLOC_MAX_SEGMENTS 4096

int bsg_price_batch_noalloc(const float* sptprice, const float* strike,
                            const float* rate, const float* volatility,
                            const float* otime, const int32_t* otype, float* prices,
                            size_t pool_len, const bsg_segment* segs, size_t nseg,
                            void* stream, unsigned flags);

/* ---- accuracy report ---------------------------------------------------
 * Compares FP32 prices (device) with the FP64 oracle evaluated on the same
 * device inputs, bucketed by |d1| (FP64) against the ascending bucket edges
 * edges[0..nbuckets] (an option with |d1| outside [edges[0], edges[nbuckets])
 * lands in the first / last bucket).  Relative error uses |oracle| with a
 * floor of rel_floor. */
typedef struct bsg_err_bucket {
    uint64_t count;
    double max_abs;
    double sum_sq_abs;
    double max_rel;
    double max_price;
} bsg_err_bucket;

#define BSG_MAX_ERR_BUCKETS 32

int bsg_error_report(bsg_ctx* ctx, const float* sptprice, const float* strike,
                     const float* rate, const float* volatility,
                     const float* otime, const int32_t* otype,
                     const float* prices, size_t n, const double* edges,
                     int nbuckets, double rel_floor, bsg_err_bucket* out);

/* ---- serving -----------------------------------------------------------
 * A request loop that admits pricing requests of any size while others are
 * on the GPU.  Admission is by a device-memory budget: a request holds 28
 * bytes per option of a resident device pool from admission to completion,
 * and waits in FIFO order while the pool or every batch slot is busy.  All
 * requests admitted since the last launch are coalesced into one batch: one
 * kernel gathers their inputs from pinned host memory into the pool, the
 * persistent batch kernel prices them, one kernel writes the prices back to
 * each request's host output.  Up to max_inflight batches overlap on the
 * GPU (one stream each).  With fused = 1 the three steps are one kernel.
 * With fused = 2 one persistent kernel keeps running instead: each admitted
 * request is published into a ring in pinned host memory that the GPU's
 * blocks take tiles from (no launch, copy or event per request); the kernel
 * exits after 5 ms without work and is relaunched when work arrives.  It
 * needs host-native atomics (NVLink-C2C; else BSG_ERR_NOT_SUPPORTED) and
 * takes requests of up to 4095 x 2048 options (else BSG_ERR_CAPACITY).
 * With plain = 1 the loop instead prices one request
 * at a time with per-array copies and one plain map launch (the baseline).
 * Request arrays are host memory; pinned memory (bsg_host_alloc or
 * cudaHostRegister) is required for the batched path and recommended for the
 * plain path.  A request's result is bit-identical alone and in any mix. */
typedef struct bsg_server bsg_server;

typedef struct bsg_server_config {
    int device;
    size_t budget_bytes;      /* device pool for admitted requests (28 B/option) */
    int max_inflight;         /* batches on the GPU at once, 1..16 */
    size_t max_batch_options; /* cap per batch (0 = the whole pool) */
    int max_batch_requests;   /* cap per batch, 1..65536 (0 = 4096) */
    int plain;                /* 1 = one plain launch per request, serially */
    unsigned flags;           /* BSG_MODE_* */
    double batch_timeout_s;   /* bound on waiting for one batch (0 = 30 s) */
    int fused;                /* 1 = one kernel per batch reads the inputs from
                                 host memory, prices them and writes the prices
                                 back (the pool then only accounts the budget);
                                 2 = the persistent kernel (no device pool);
                                 0 = gather into the pool, price, scatter */
    int persistent_blocks;    /* fused = 2: blocks of the persistent kernel,
                                 8..4096 (0 = SMs x min(occupancy, 3)) */
    int persistent_window;    /* fused = 2: how many of the oldest requests
                                 the blocks share at once, 1..16 (0 = the
                                 default; 1 = the oldest request's tiles first) */
} bsg_server_config;

typedef struct bsg_request {
    const float* sptprice;
    const float* strike;
    const float* rate;
    const float* volatility;
    const float* otime;
    const int32_t* otype;
    float* prices;
    size_t n;
} bsg_request;

typedef struct bsg_server_stats {
    uint64_t submitted, completed, cancelled, failed;
    uint64_t batches;          /* batches launched (persistent path: requests published) */
    uint64_t kernel_launches;  /* persistent path: launches of the persistent kernel */
    uint64_t options_priced;
    uint64_t max_batch_requests_seen;
    uint64_t queued, inflight_requests;
} bsg_server_stats;

int bsg_server_create(bsg_server** out, const bsg_server_config* cfg);
/* Destroys the loop: queued requests are cancelled, in-flight ones finish. */
void bsg_server_destroy(bsg_server* srv);
/* Registers host memory [ptr, ptr + bytes) for request arrays of the batched
 * path (pins it with cudaHostRegister unless it is already pinned).  Every
 * array of a batched request must lie inside one registered range: the GPU
 * reads inputs and writes prices there directly over the host link. */
int bsg_server_register(bsg_server* srv, void* ptr, size_t bytes);
/* Enqueues a request (non-blocking).  BSG_ERR_BUDGET if it can never fit.
 * A request of n == 0 options completes at once with BSG_OK. */
int bsg_server_submit(bsg_server* srv, const bsg_request* req, uint64_t* id);
/* Waits up to timeout_s (< 0: no limit) for request id.  Returns its final
 * status (BSG_OK priced, BSG_ERR_CANCELLED, BSG_ERR_TIMEOUT for a batch that
 * overran batch_timeout_s, ...) and releases it, or BSG_ERR_TIMEOUT while it
 * is still pending (it stays pending).  latency_s (optional): submit to
 * completion. */
int bsg_server_wait(bsg_server* srv, uint64_t id, double timeout_s, double* latency_s);
/* Cancels a request that is still queued; BSG_ERR_STATE once admitted. */
int bsg_server_cancel(bsg_server* srv, uint64_t id);
/* Holds (1) or resumes (0) admission; queued requests stay queued. */
int bsg_server_pause(bsg_server* srv, int paused);
int bsg_server_get_stats(bsg_server* srv, bsg_server_stats* out);

/* Open-loop trace: Poisson arrivals at rate_per_s for duration_s, request
 * sizes log-uniform in [min_n, max_n], each request a slice of the caller's
 * pinned host pool (5 float arrays + otype, and a prices array, each of
 * pool_n options) at a seeded offset.  Latency runs from each request's
 * scheduled arrival to its completion.  Latencies of completed requests are
 * written to latencies_out (capacity latencies_cap; may be NULL). */
typedef struct bsg_trace_config {
    double rate_per_s;
    double duration_s;
    size_t min_n, max_n;
    uint64_t seed;
    const float* sptprice;
    const float* strike;
    const float* rate;
    const float* volatility;
    const float* otime;
    const int32_t* otype;
    float* prices;
    size_t pool_n;
    double drain_timeout_s; /* bound on waiting for the last requests (0 = 60 s) */
} bsg_trace_config;

typedef struct bsg_trace_result {
    uint64_t requests, completed, failed;
    uint64_t options;
    double wall_s;          /* first arrival to last completion */
    double options_per_s, requests_per_s;
    double p50_s, p99_s, p999_s, max_s, mean_s;
    double mean_batch_requests;
    uint64_t batches;
    double late_submit_max_s; /* how far behind schedule the submitter fell
                                 (BSG_TRACE_DEBUG=1 prints which request) */
} bsg_trace_result;

int bsg_serve_trace(const bsg_server_config* cfg, const bsg_trace_config* trace,
                    bsg_trace_result* out, double* latencies_out, size_t latencies_cap);

/* ---- swaptions (HJM Monte Carlo) --------------------------------------
 * P3ARSEC's swaptions application: each swaption priced by Monte Carlo
 * simulation of forward-rate paths under a multi-factor HJM model
 * (parsec-ff/pkgs/apps/swaptions/src/HJM_Swaption_Blocking.cpp:19-223),
 * one swaption per iteration of a FastFlow ParallelFor
 * (HJM_Securities.cpp:312-323).  The reference tree holds the driver but
 * not the model core, so the model here is the published discrete HJM
 * model (time-to-maturity parameterisation, the drift that makes
 * discounted bonds martingales) and the paths' variates come from a
 * counter-based generator keyed by (seed, trial): prices agree with the
 * reference's in distribution, not trial for trial.  Double precision
 * throughout, as the reference's FTYPE. */
typedef struct bsg_swaption {
    double strike;           /* dStrike */
    double compounding;      /* dCompounding: 0 = the strike is continuously compounded */
    double maturity;         /* dMaturity: years to the option's expiry */
    double tenor;            /* dTenor: years of the underlying swap */
    double payment_interval; /* dPaymentInterval: years between swap payments */
    double years;            /* dYears: horizon of the HJM grid */
    int n_steps;             /* iN: grid points, 2..32 */
    int n_factors;           /* iFactors: volatility factors, 1..8 */
    const double* yield;     /* n_steps continuously compounded yields */
    const double* factors;   /* n_factors x (n_steps - 1) vols, row-major: factor
                                k's vol of the forward m + 1 steps from maturity */
    uint64_t seed;           /* the paths' random stream (iRndSeed) */
} bsg_swaption;

/* Prices n swaptions with `trials` paths each (2..2^40) in one launch:
 * price[i] = mean discounted payoff max(V - 1, 0) D, std_err[i] (optional)
 * = its standard error, both as the reference computes them
 * (HJM_Swaption_Blocking.cpp:191-214).  Host arrays; the call returns when
 * the results are in.  Deterministic: the same inputs give the same bits.
 * BSG_ERR_INVALID_ARG names the first swaption whose maturity, tenor or
 * payment interval does not fit its grid. */
int bsg_price_swaptions(bsg_ctx* ctx, const bsg_swaption* swaptions, size_t n,
                        uint64_t trials, double* price, double* std_err);

/* The normal variates the swaption kernel draws, for given random words:
 * words[4 i .. 4 i + 3] (host array) -> z[2 i], z[2 i + 1] (host array), by
 * the device's Box-Muller transform (u1 from words 0-1, u2 from words 2-3,
 * u = (2k + 1) 2^-53 with k = the top 20 bits of the first word and all of
 * the second).  For checking the transform against a host evaluation. */
int bsg_swaption_normals(bsg_ctx* ctx, const uint32_t* words, size_t n_pairs, double* z);

/* The reference's per-swaption signature (HJM_Swaption_Blocking.cpp:19-41;
 * FTYPE = double) on the default context of device 0: pdSwaptionPrice[0] =
 * price, [1] = standard error.  Returns 1 on success as the reference does,
 * else a bsg_status.  BLOCKSIZE and tid are accepted and unused. */
int bsg_HJM_Swaption_Blocking(double* pdSwaptionPrice, double dStrike, double dCompounding,
                              double dMaturity, double dTenor, double dPaymentInterval,
                              int iN, int iFactors, double dYears, double* pdYield,
                              double** ppdFactors, long iRndSeed, long lTrials,
                              int BLOCKSIZE, int tid);

/* ---- the reference's file formats (host code) --------------------------
 * Input, blackscholes.c:695-739: a count ("%i"), then per option
 * "%f %f %f %f %f %f %c %f %f" = s strike r divq v t OptionType divs
 * DGrefval; otype = 1 for 'P', else 0 (:760).  Floats convert as the
 * reference's fscanf does (strtof), so arrays are bit-identical; parsing runs
 * on nthreads threads (0 = all cores).  Output, :923-947: "%i\n" then
 * "%.18f\n" per price, byte-identical to the reference's fprintf.  A bsg_book
 * owns one 256-byte-aligned host allocation (release with bsg_book_free). */
typedef struct bsg_book {
    size_t n;
    float* sptprice;
    float* strike;
    float* rate;
    float* volatility;
    float* otime;
    int32_t* otype;
    float* dgrefval;
    void* mem_; /* owned allocation */
} bsg_book;

int bsg_read_parsec(const char* path, int nthreads, bsg_book* out);
int bsg_parse_parsec(const char* text, size_t len, int nthreads, bsg_book* out);
void bsg_book_free(bsg_book* book);
int bsg_write_parsec_prices(const char* path, const float* prices, size_t n, int nthreads);
/* The output text in memory (release with bsg_text_free). */
int bsg_format_prices(const float* prices, size_t n, int nthreads, char** text, size_t* len);
void bsg_text_free(char* text);
/* An input file in the same format (floats as "%.9g", which round-trips
 * through "%f"; divq = divs = 0; DGrefval from the book, 0 if NULL). */
int bsg_write_parsec_input(const char* path, const bsg_book* book, int nthreads);
/* Binary SoA file ("BSGSOA01", uint64 n, the seven arrays). */
int bsg_write_soa(const char* path, const bsg_book* book);
int bsg_read_soa(const char* path, bsg_book* out);

/* ---- tuning ------------------------------------------------------------
 * The plain map is a family of kernels: vector width per thread, block size,
 * grid size, load path and, for the resident-prefix load path, the prefix
 * size.  bsg_autotune times the candidates on the context's device for n
 * options and makes the fastest the context's choice: every shape over 5
 * passes; then the prefix sizes 4..24 32nds of the L2 for the best
 * resident-prefix shape over 25 passes; then the four fastest shapes over
 * BSG_NUM_RUNS passes, three times each, the best time of each.  The result is cached in the file named by
 * $BSG_TUNE_CACHE (if set) per (device, size bucket). */
typedef struct bsg_tune {
    int vec_per_thread; /* float4 groups per thread per tile: 1, 2 or 4 */
    int block;          /* threads per block: 128, 256 or 512 */
    int blocks_per_sm;  /* grid = blocks_per_sm * SM count; 0 = one block per tile */
    int load_path;      /* 0 = LDG.128 non-coherent, 1 = LDG.128 evict-first,
                           2 = LDG.256 non-coherent (8 options per load),
                           3, 4, 5 = TMA bulk copies into a shared-memory
                               ring of 3 x 48 KB (1 CTA per SM), 4 x 24 KB
                               (2 per SM) or 3 x 24 KB (3 per SM); block and
                               grid are then fixed,
                           6 = LDG.256 evict-first (vec_per_thread 1 or 2),
                           7 = LDG.256 and STG.256 with the book's first
                               options (resident_32nds of the L2 at 28 bytes
                               each) evict-last, the rest evict-first: that
                               prefix stays in L2 across passes,
                           8 = LDG.256 and STG.256 with the default L2
                               policy, every other pass walking the book
                               from its last tile to its first: each pass
                               starts on the lines the previous one touched
                               last (vec_per_thread 1 or 2) */
    int pdl;            /* 1 = programmatic dependent launch between passes */
    int resident_32nds; /* load path 7: size of the resident prefix in 32nds
                           of the device's L2, 1..24; 0 = 15 */
} bsg_tune;

int bsg_autotune(bsg_ctx* ctx, size_t n, bsg_tune* out);

/* Self-test of the device-side failure detection: launches the staged map
 * kernel with every mbarrier expecting more bytes than its copies deliver,
 * so each of its waits runs out after limit_s (0 < limit_s <= 10) of GPU
 * time; the kernel records the expiry, lets its copies land and returns.
 * Expected result: BSG_ERR_TIMEOUT, the context still usable afterwards.
 * elapsed_s (optional): host time of the call. */
int bsg_selftest_wait_timeout(bsg_ctx* ctx, double limit_s, double* elapsed_s);

/* Self-test of the debug guards (contexts created with BSG_DEBUG set):
 * overwrites the last guard word after the resident price array (inside the
 * context's own allocation), runs the post-call check, then restores the
 * word.  Expected result: BSG_ERR_STATE with the word named by
 * bsg_last_error(); BSG_ERR_NOT_SUPPORTED without BSG_DEBUG. */
int bsg_selftest_guard(bsg_ctx* ctx);
int bsg_get_tune(const bsg_ctx* ctx, bsg_tune* out);
int bsg_set_tune(bsg_ctx* ctx, const bsg_tune* tune);

#ifdef __cplusplus
}
#endif
#endif /* BSG_H */
