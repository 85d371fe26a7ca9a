// bsg_swaptions.cu -- sm_103a kernels of the swaption Monte Carlo (HJM).
//
// P3ARSEC's swaptions application prices every swaption with
// HJM_Swaption_Blocking (parsec-ff/pkgs/apps/swaptions/src/
// HJM_Swaption_Blocking.cpp:19-223), one swaption per FastFlow worker
// iteration (HJM_Securities.cpp:312-323), trials in blocks on one core.  Here
// one launch prices every swaption: a grid of (trial chunk, swaption) blocks,
// one path per thread at a time, in double precision as the reference's
// FTYPE.
//
// Per path (the driver's arithmetic, HJM_Swaption_Blocking.cpp:160-204, on
// a discrete HJM model in the time-to-maturity parameterisation):
//   f(t_{i+1}, t_{i+1+m}) = f(t_i, t_{i+1+m}) + mu[m] h + sqrt(h) sum_k v_k[m] z_ik
//   D     = exp(-h sum_{i<s} f(t_i, t_i))               discount to maturity t_s
//   V     = sum_l pay[l] exp(-h sum_{m<l} f(t_s, t_{s+m}))   fixed leg at t_s
//   price = mean of max(V - 1, 0) D,  error = the reference's standard error
// with mu[m] = (h/2) sum_k (S_k(m)^2 - S_k(m-1)^2) (S_k: running sums of
// factor k's vols), the drift that makes discounted bonds martingales.
//
// Work that cannot reach the payoff is not done: rows of the path after the
// swaption's maturity t_s (the reference simulates all n_steps - 1 of them),
// the entries of each row that no payment date of the swap reads, and the
// discount factors of swap dates without a payment.  The variates of the
// rows that are simulated are the same ones: each is drawn from a
// counter-based generator (Philox4x32-10, Salmon et al., SC'11) keyed by
// (seed, trial, index) and turned normal by Box-Muller (bsg_swmath.h:
// table-driven -2 ln u and sin/cos(2 pi u) from the uniforms' bits), so the
// prices equal those of a full-path simulation with the same stream.  The
// kernel is bound by GB300's FP64 rate; the trimming and the table-driven
// transform and exp (bsg_swmath.h) halve its double-precision work per path.
//
// Reduction: each block reduces its paths' sums (sum and sum of squares of
// the discounted payoff) in a fixed order and writes one partial; a second
// kernel adds a swaption's partials in a fixed order.  Results do not depend
// on scheduling: two runs give the same bits.
#include "bsg_internal.h"
#include "bsg_swmath.h"

#include <math.h>

#include <algorithm>

namespace bsg {

namespace {

constexpr int kSwThreads = 256;

__device__ __forceinline__ void philox4x32_10(uint32_t x0, uint32_t x1, uint32_t x2, uint32_t x3,
                                              uint32_t k0, uint32_t k1, uint32_t out[4]) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t lo0 = 0xD2511F53u * x0, hi0 = __umulhi(0xD2511F53u, x0);
        const uint32_t lo1 = 0xCD9E8D57u * x2, hi1 = __umulhi(0xCD9E8D57u, x2);
        const uint32_t y0 = hi1 ^ x1 ^ k0, y2 = hi0 ^ x3 ^ k1;
        x0 = y0;
        x1 = lo1;
        x2 = y2;
        x3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = x0;
    out[1] = x1;
    out[2] = x2;
    out[3] = x3;
}

// Normal variates 2j and 2j + 1 of trial t: Box-Muller on the uniforms of
// the Philox block (seed, t, j), evaluated from their bits (bsg_swmath.h).
__device__ __forceinline__ void normal_pair(const bsg_sw::Tables& tab, uint64_t seed, uint64_t t,
                                            uint32_t j, double& z0, double& z1) {
    uint32_t x[4];
    philox4x32_10((uint32_t)t, (uint32_t)(t >> 32), j, 0u, (uint32_t)seed, (uint32_t)(seed >> 32), x);
    bsg_sw::normal_pair(tab, x[0], x[1], x[2], x[3], &z0, &z1);
}

__device__ const bsg_sw::Tables kSwTables = BSG_SW_TABLES;

// Copies the tables of bsg_swmath.h into shared memory (all threads of the block).
__device__ __forceinline__ void load_tables(bsg_sw::Tables& dst) {
    const double2* src = reinterpret_cast<const double2*>(&kSwTables);
    double2* d = reinterpret_cast<double2*>(&dst);
    for (int i = threadIdx.x; i < (int)(sizeof(bsg_sw::Tables) / sizeof(double2)); i += blockDim.x)
        d[i] = src[i];
}

// Per-swaption constants in shared memory: the forward curve, the drift
// times h, the vols times sqrt(h), the swap payments.
template <int MAXN>
struct SwShared {
    double fwd[MAXN];
    double muh[MAXN];
    double vol[kSwMaxFactors][MAXN];
    double pay[MAXN];
    double red[2][kSwThreads / 32];
    bsg_sw::Tables nt;
};

// Paths q * kSwThreads + threadIdx.x (q < per_thread) of one block, with the
// path rows cut to the NEED entries that reach the payoff (row i of the
// reference's path computes all n - 1 - i; the others never reach a
// payment date before the swap's last, so the price is the same).
template <int MAXN, int NEED>
__device__ __forceinline__ void price_paths(const SwParams& p, const SwShared<MAXN>& sh, uint64_t base,
                                            int per_thread, uint64_t trials, double& sum,
                                            double& sum_sq) {
    const int s = p.start, nf = p.n_factors, last = p.swap_points;
    const double h = p.h;
    for (int q = 0; q < per_thread; ++q) {
        const uint64_t t = base + (uint64_t)q * kSwThreads + threadIdx.x;
        if (t >= trials) break;
        double f[NEED + 1];
#pragma unroll
        for (int m = 0; m <= NEED; ++m) f[m] = sh.fwd[m];
        double acc = 0.0, zc[2] = {0.0, 0.0};
        int zi = 0;  // index of the next normal variate of this trial
        for (int i = 0; i < s; ++i) {
            acc += f[0];
            double shock[NEED];
#pragma unroll
            for (int m = 0; m < NEED; ++m) shock[m] = 0.0;
            for (int k = 0; k < nf; ++k, ++zi) {
                if ((zi & 1) == 0) normal_pair(sh.nt, p.seed, t, (uint32_t)(zi >> 1), zc[0], zc[1]);
                const double z = zc[zi & 1];
#pragma unroll
                for (int m = 0; m < NEED; ++m) shock[m] = __fma_rn(sh.vol[k][m], z, shock[m]);
            }
            // row i + 1 from row i (entries at or past NEED - i are never read)
#pragma unroll
            for (int m = 0; m < NEED; ++m) f[m] = f[m + 1] + sh.muh[m] + shock[m];
        }
        const double disc = bsg_sw::exp_(sh.nt, -acc * h);
        double fixed = 0.0, accs = 0.0;
#pragma unroll
        for (int l = 0; l <= NEED; ++l) {
            if (l <= last && sh.pay[l] != 0.0) fixed += sh.pay[l] * bsg_sw::exp_(sh.nt, -accs * h);
            accs += f[l];
        }
        const double payoff = fixed - 1.0 > 0.0 ? fixed - 1.0 : 0.0;
        const double dp = payoff * disc;
        sum += dp;
        sum_sq += dp * dp;
    }
}

// One block: paths [chunk * per_block, ...) of swaption blockIdx.y.
template <int MAXN>
__global__ void __launch_bounds__(kSwThreads, MAXN <= 12 ? 2 : 1) swaption_paths_kernel(const SwParams* __restrict__ prm,
                                                                    uint64_t trials, int per_thread,
                                                                    double* __restrict__ partial) {
    __shared__ SwShared<MAXN> sh;
    const SwParams& p = prm[blockIdx.y];
    const int n = p.n_steps, nf = p.n_factors;
    const double h = p.h;
    // set-up, the same in every block of the swaption: forward curve from the
    // yields, drift from the vols, payments (HJM_Swaption_Blocking.cpp:132-140)
    load_tables(sh.nt);
    if (threadIdx.x < MAXN) {
        const int i = threadIdx.x;
        sh.fwd[i] = i == 0 ? p.yield[0]
                           : (i < n ? (double)(i + 1) * p.yield[i] - (double)i * p.yield[i - 1] : 0.0);
        double pay = 0.0;
        if (i < p.swap_len && i >= p.freq && i <= p.swap_points && (i % p.freq) == 0)
            pay = i == p.swap_points ? exp(p.strike_cont * p.payment_interval)
                                     : exp(p.strike_cont * p.payment_interval) - 1;
        sh.pay[i] = pay;
        double mu = 0.0;
        for (int k = 0; k < nf; ++k) {
            double s_prev = 0.0;
            for (int m = 0; m < i && m < n - 1; ++m) s_prev += p.vol[k][m];
            const double vk = i < n - 1 ? p.vol[k][i] : 0.0;
            mu += h * vk * (s_prev + 0.5 * vk);
            sh.vol[k][i] = vk * p.sqh;
        }
        sh.muh[i] = mu * h;
    }
    __syncthreads();
    const uint64_t base = (uint64_t)blockIdx.x * per_thread * kSwThreads;
    double sum = 0.0, sum_sq = 0.0;
    // rows of the path that reach the payoff: row i needs entries
    // m < swap_points + start - 1 - i (the last payment's discount reads
    // f[0 .. swap_points - 1] of row start); swap_points + start <= n - 1
    switch (p.swap_points + p.start - 1) {
        case 1: price_paths<MAXN, 1>(p, sh, base, per_thread, trials, sum, sum_sq); break;
        case 2: price_paths<MAXN, 2>(p, sh, base, per_thread, trials, sum, sum_sq); break;
        case 3: price_paths<MAXN, 3>(p, sh, base, per_thread, trials, sum, sum_sq); break;
        case 4: price_paths<MAXN, 4>(p, sh, base, per_thread, trials, sum, sum_sq); break;
        case 5: price_paths<MAXN, 5>(p, sh, base, per_thread, trials, sum, sum_sq); break;
        case 6: price_paths<MAXN, 6>(p, sh, base, per_thread, trials, sum, sum_sq); break;
        case 7: price_paths<MAXN, 7>(p, sh, base, per_thread, trials, sum, sum_sq); break;
        case 8: price_paths<MAXN, 8>(p, sh, base, per_thread, trials, sum, sum_sq); break;
        case 9: price_paths<MAXN, 9>(p, sh, base, per_thread, trials, sum, sum_sq); break;
        case 10: price_paths<MAXN, 10>(p, sh, base, per_thread, trials, sum, sum_sq); break;
        default: price_paths<MAXN, MAXN - 1>(p, sh, base, per_thread, trials, sum, sum_sq); break;
    }
    // block reduction in a fixed order
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_down_sync(0xffffffffu, sum, o);
        sum_sq += __shfl_down_sync(0xffffffffu, sum_sq, o);
    }
    if ((threadIdx.x & 31) == 0) {
        sh.red[0][threadIdx.x >> 5] = sum;
        sh.red[1][threadIdx.x >> 5] = sum_sq;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < kSwThreads / 32; ++w) {
            a += sh.red[0][w];
            b += sh.red[1][w];
        }
        partial[2 * ((size_t)blockIdx.y * gridDim.x + blockIdx.x)] = a;
        partial[2 * ((size_t)blockIdx.y * gridDim.x + blockIdx.x) + 1] = b;
    }
}

// One block per swaption: its chunks' partials in a fixed order, then the
// mean and the reference's standard error (HJM_Swaption_Blocking.cpp:212-214).
__global__ void __launch_bounds__(kSwThreads) swaption_reduce_kernel(const double* __restrict__ partial,
                                                                     int chunks, uint64_t trials,
                                                                     double* __restrict__ out) {
    __shared__ double sa[kSwThreads], sb[kSwThreads];
    double a = 0.0, b = 0.0;
    const double* p = partial + 2 * (size_t)blockIdx.x * chunks;
    for (int c = threadIdx.x; c < chunks; c += kSwThreads) {
        a += p[2 * c];
        b += p[2 * c + 1];
    }
    sa[threadIdx.x] = a;
    sb[threadIdx.x] = b;
    __syncthreads();
    for (int w = kSwThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            sa[threadIdx.x] += sa[threadIdx.x + w];
            sb[threadIdx.x] += sb[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double m = (double)trials, sum = sa[0], sum_sq = sb[0];
        out[2 * blockIdx.x] = sum / m;
        out[2 * blockIdx.x + 1] = sqrt((sum_sq - sum * sum / m) / (m - 1.0)) / sqrt(m);
    }
}

__global__ void __launch_bounds__(kSwThreads) swaption_normals_kernel(const uint32_t* __restrict__ words,
                                                                      uint64_t n, double* __restrict__ z) {
    __shared__ bsg_sw::Tables nt;
    load_tables(nt);
    __syncthreads();
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        bsg_sw::normal_pair(nt, words[4 * i], words[4 * i + 1], words[4 * i + 2], words[4 * i + 3],
                            &z[2 * i], &z[2 * i + 1]);
}

}  // namespace

cudaError_t launch_swaption_normals(const uint32_t* words, uint64_t n, double* z, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    const uint64_t blocks = std::min<uint64_t>((n + kSwThreads - 1) / kSwThreads, 4096);
    swaption_normals_kernel<<<(unsigned)blocks, kSwThreads, 0, st>>>(words, n, z);
    return cudaGetLastError();
}

int swaption_chunks(uint64_t trials, int per_thread) {
    const uint64_t per_block = (uint64_t)per_thread * kSwThreads;
    return (int)((trials + per_block - 1) / per_block);
}

cudaError_t launch_swaptions(const SwParams* prm, int nsw, int max_steps, uint64_t trials,
                             int per_thread, double* partial, double* out, cudaStream_t st) {
    if (nsw <= 0 || trials < 2 || per_thread < 1) return cudaErrorInvalidValue;
    const int chunks = swaption_chunks(trials, per_thread);
    if (nsw > 65535) return cudaErrorInvalidValue;
    const dim3 grid((unsigned)chunks, (unsigned)nsw);
    if (max_steps <= 12)
        swaption_paths_kernel<12><<<grid, kSwThreads, 0, st>>>(prm, trials, per_thread, partial);
    else
        swaption_paths_kernel<kSwMaxSteps><<<grid, kSwThreads, 0, st>>>(prm, trials, per_thread, partial);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    swaption_reduce_kernel<<<(unsigned)nsw, kSwThreads, 0, st>>>(partial, chunks, trials, out);
    return cudaGetLastError();
}

}  // namespace bsg
