// Test harness for include/bsg_map.cuh (compiled by tests/test_map_skeleton.py).
// Instantiates the generic map with the Black-Scholes price (must equal
// bsg_price_soa bit for bit), an AXPY and a mixed-type map.
#include "bsg_map.cuh"
#include "bsg_math.cuh"

struct BsFast {
    __device__ float operator()(float s, float k, float r, float v, float t, int32_t ot) const {
        return bsg::price_fast(s, k, r, v, t, ot);
    }
};

struct Axpy {
    float a;
    __device__ float operator()(float x, float y) const { return __fmaf_rn(a, x, y); }
};

struct Mixed {
    __device__ double operator()(int32_t i, float f, double d) const {
        return __dadd_rn((double)i, __dmul_rn((double)f, d));
    }
};

extern "C" int skel_bs(int64_t n, const float* s, const float* k, const float* r, const float* v,
                       const float* t, const int32_t* ot, float* out, int pdl, int runs) {
    bsg::MapShape sh;
    sh.pdl = pdl != 0;
    for (int j = 0; j < runs; ++j) {
        cudaError_t e = bsg::map_shaped(sh, 0, BsFast{}, n, out, s, k, r, v, t, ot);
        if (e != cudaSuccess) return (int)e;
    }
    return (int)cudaDeviceSynchronize();
}

extern "C" int skel_axpy(int64_t n, float a, const float* x, const float* y, float* out) {
    cudaError_t e = bsg::map(0, Axpy{a}, n, out, x, y);
    if (e != cudaSuccess) return (int)e;
    return (int)cudaDeviceSynchronize();
}

extern "C" int skel_mixed(int64_t n, const int32_t* i, const float* f, const double* d, double* out) {
    cudaError_t e = bsg::map(0, Mixed{}, n, out, i, f, d);
    if (e != cudaSuccess) return (int)e;
    return (int)cudaDeviceSynchronize();
}
