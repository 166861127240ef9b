// Shared device helpers for the GB300 tomography kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define ACU_HD __host__ __device__ __forceinline__

namespace acu {

// A group of V slices processed by one thread.  Arrays in "lane layout" hold
// the V slices of a group interleaved: element (group g, position i, lane v)
// sits at ((g * npos) + i) * V + v, so one thread moves a group with a
// single vector access (V = 4: 16-byte float4).
template <typename Real, int V>
struct Lanes {
    Real v[V];
};

template <typename Real, int V>
__device__ __forceinline__ Lanes<Real, V> ld_lanes(const Real* __restrict__ p)
{
    Lanes<Real, V> r;
    if constexpr (V == 4 && sizeof(Real) == 4) {
        float4 t = __ldg(reinterpret_cast<const float4*>(p));
        r.v[0] = t.x; r.v[1] = t.y; r.v[2] = t.z; r.v[3] = t.w;
    } else if constexpr (V == 2 && sizeof(Real) == 8) {
        double2 t = __ldg(reinterpret_cast<const double2*>(p));
        r.v[0] = t.x; r.v[1] = t.y;
    } else if constexpr (V == 2 && sizeof(Real) == 4) {
        float2 t = __ldg(reinterpret_cast<const float2*>(p));
        r.v[0] = t.x; r.v[1] = t.y;
    } else {
#pragma unroll
        for (int i = 0; i < V; ++i) r.v[i] = __ldg(p + i);
    }
    return r;
}

// Plain (coherent) load for buffers written earlier in the same kernel chain.
template <typename Real, int V>
__device__ __forceinline__ Lanes<Real, V> ld_lanes_rw(const Real* p)
{
    Lanes<Real, V> r;
    if constexpr (V == 4 && sizeof(Real) == 4) {
        float4 t = *reinterpret_cast<const float4*>(p);
        r.v[0] = t.x; r.v[1] = t.y; r.v[2] = t.z; r.v[3] = t.w;
    } else if constexpr (V == 2 && sizeof(Real) == 8) {
        double2 t = *reinterpret_cast<const double2*>(p);
        r.v[0] = t.x; r.v[1] = t.y;
    } else {
#pragma unroll
        for (int i = 0; i < V; ++i) r.v[i] = p[i];
    }
    return r;
}

template <typename Real, int V>
__device__ __forceinline__ void st_lanes(Real* p, const Lanes<Real, V>& r)
{
    if constexpr (V == 4 && sizeof(Real) == 4) {
        *reinterpret_cast<float4*>(p) = make_float4(r.v[0], r.v[1], r.v[2], r.v[3]);
    } else if constexpr (V == 2 && sizeof(Real) == 8) {
        *reinterpret_cast<double2*>(p) = make_double2(r.v[0], r.v[1]);
    } else {
#pragma unroll
        for (int i = 0; i < V; ++i) p[i] = r.v[i];
    }
}

// Round-to-nearest arithmetic that the compiler may not contract into FMA:
// coordinates are evaluated in the reference's operation order so that the
// interpolation cells chosen match the reference's single-precision ones.
ACU_HD float mul_rn(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
ACU_HD float add_rn(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
ACU_HD float sub_rn(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
ACU_HD double mul_rn(double a, double b)
{
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
ACU_HD double add_rn(double a, double b)
{
#ifdef __CUDA_ARCH__
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
ACU_HD double sub_rn(double a, double b)
{
#ifdef __CUDA_ARCH__
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}

__device__ __forceinline__ float rfloor(float x) { return floorf(x); }
__device__ __forceinline__ double rfloor(double x) { return floor(x); }

// Block-wide sum of one double per thread; result valid in thread 0.
// blockDim.x * blockDim.y must be a multiple of 32 and at most 1024.
__device__ __forceinline__ double block_sum(double v, double* sh /* >= 32 */)
{
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    const int nthreads = blockDim.x * blockDim.y;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((tid & 31) == 0) sh[tid >> 5] = v;
    __syncthreads();
    double r = 0.0;
    if (tid < 32) {
        r = (tid < (nthreads >> 5)) ? sh[tid] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    }
    return r;
}

}  // namespace acu
