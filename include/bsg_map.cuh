// bsg_map.cuh -- a generic elementwise map for sm_103a (header only, CUDA C++).
//
//     out[i] = f(in_0[i], in_1[i], ..., in_k[i])   for i < n
//
// The GB300 counterpart of SkePU2's Map<arity> skeleton and its CUDA
// back-end (parsec-ff/pkgs/libs/skepu2/include/skepu2/map.hpp;
// backend/impl/map/map_cu.inl:15-57, kernel template
// clang_precompiler/map_cu.cpp:9-22), which launches a scalar grid-stride
// loop.  This skeleton is the one the Black-Scholes map runs on:
//  * each thread handles groups of 4 consecutive elements; every input and
//    the output are read and written with 16-byte vector accesses (two for
//    8-byte types) when all pointers are 16-byte aligned, scalar otherwise;
//  * persistent grid of blocks_per_sm x the SM count, grid-stride over groups;
//  * optional programmatic dependent launch, so back-to-back maps on one
//    stream overlap one's tail with the next one's ramp-up (the kernel waits
//    for the previous grid only after its own stores).
// f is any callable usable in device code (a functor with a __device__
// operator(), or an extended __device__ lambda with nvcc --extended-lambda).
// Element types of 4 or 8 bytes use vector accesses; others are scalar.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstring>

namespace bsg {

struct MapShape {
    int block = 256;         // threads per block
    int blocks_per_sm = 4;   // persistent grid = blocks_per_sm x SMs
    bool pdl = false;        // programmatic dependent launch
};

namespace map_detail {

template <typename T>
struct Lane4 {
    T v[4];
};

template <bool VEC, typename T>
__device__ __forceinline__ Lane4<T> load4(const T* __restrict__ p, int64_t i) {
    Lane4<T> r;
    if constexpr (VEC && sizeof(T) == 4) {
        const uint4 u = __ldg(reinterpret_cast<const uint4*>(p + i));
        memcpy(r.v, &u, 16);
    } else if constexpr (VEC && sizeof(T) == 8) {
        const ulonglong2 a = __ldg(reinterpret_cast<const ulonglong2*>(p + i));
        const ulonglong2 b = __ldg(reinterpret_cast<const ulonglong2*>(p + i + 2));
        memcpy(r.v, &a, 16);
        memcpy(r.v + 2, &b, 16);
    } else {
#pragma unroll
        for (int e = 0; e < 4; ++e) r.v[e] = p[i + e];
    }
    return r;
}

template <bool VEC, typename T>
__device__ __forceinline__ void store4(T* __restrict__ p, int64_t i, const T (&x)[4]) {
    if constexpr (VEC && sizeof(T) == 4) {
        uint4 u;
        memcpy(&u, x, 16);
        __stcs(reinterpret_cast<uint4*>(p + i), u);
    } else if constexpr (VEC && sizeof(T) == 8) {
        ulonglong2 a, b;
        memcpy(&a, x, 16);
        memcpy(&b, x + 2, 16);
        __stcs(reinterpret_cast<ulonglong2*>(p + i), a);
        __stcs(reinterpret_cast<ulonglong2*>(p + i + 2), b);
    } else {
#pragma unroll
        for (int e = 0; e < 4; ++e) p[i + e] = x[e];
    }
}

template <typename F, typename Out, typename... In>
__device__ __forceinline__ void apply4(const F& f, Out (&r)[4], const Lane4<In>&... lanes) {
#pragma unroll
    for (int e = 0; e < 4; ++e) r[e] = f(lanes.v[e]...);
}

template <bool VEC, typename F, typename Out, typename... In>
__global__ void map_kernel(F f, int64_t n, Out* __restrict__ out, const In* __restrict__... in) {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const int64_t groups = n / 4;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (int64_t g = tid; g < groups; g += stride) {
        Out r[4];
        apply4(f, r, load4<VEC>(in, 4 * g)...);
        store4<VEC>(out, 4 * g, r);
    }
    const int64_t i = 4 * groups + tid;
    if (i < n) out[i] = f(in[i]...);
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

inline int sm_count() {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return 1;
    return sms > 0 ? sms : 1;
}

template <typename T>
inline uintptr_t addr(const T* p) {
    return reinterpret_cast<uintptr_t>(p);
}

}  // namespace map_detail

// Launches the map on `stream` with `shape` (asynchronous; returns the
// launch status).  n <= 0 is a no-op.
template <typename F, typename Out, typename... In>
cudaError_t map_shaped(const MapShape& shape, cudaStream_t stream, const F& f, int64_t n,
                       Out* out, const In*... in) {
    static_assert(sizeof...(In) >= 1, "a map needs at least one input");
    if (n <= 0) return cudaSuccess;
    if (shape.block < 32 || shape.block > 1024 || shape.blocks_per_sm < 1)
        return cudaErrorInvalidValue;
    const uintptr_t any = map_detail::addr(out) | (map_detail::addr(in) | ...);
    const int64_t need = (n / 4 + shape.block - 1) / shape.block;
    int64_t grid = (int64_t)shape.blocks_per_sm * map_detail::sm_count();
    if (grid > need) grid = need;
    if (grid < 1) grid = 1;
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)grid);
    lc.blockDim = dim3((unsigned)shape.block);
    lc.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    lc.attrs = attr;
    lc.numAttrs = shape.pdl ? 1 : 0;
    void (*kernel)(F, int64_t, Out*, const In*...) =
        ((any & 15) == 0) ? map_detail::map_kernel<true, F, Out, In...>
                          : map_detail::map_kernel<false, F, Out, In...>;
    return cudaLaunchKernelEx(&lc, kernel, f, n, out, in...);
}

template <typename F, typename Out, typename... In>
cudaError_t map(cudaStream_t stream, const F& f, int64_t n, Out* out, const In*... in) {
    return map_shaped(MapShape{}, stream, f, n, out, in...);
}

}  // namespace bsg
