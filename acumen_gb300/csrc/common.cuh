// Shared device helpers for the GB300 tomography kernels.
#pragma once
#include <atomic>
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

// Per-thread partial of a CG reduction (an inner product or a norm).
// Double precision: an FP64 sum as before.  Single precision: the product of
// two floats is held exactly as the pair (p, fma(a, b, -p)) and the terms are
// summed in a double-float pair (two-sum, then renormalised), which is
// converted to FP64 once per thread for the FP64 block and slice sums.  GB300
// issues FP64 at a small fraction of its FP32 rate, and one FP64 multiply-add
// plus two conversions per element held these kernels to about a third of the
// HBM bandwidth; the pair keeps each term to ~2^-48 of the partial.
template <typename Real>
struct SumAcc {
    double s = 0.0;
    __device__ __forceinline__ void add_prod(double a, double b) { s += a * b; }
    __device__ __forceinline__ void add(double a) { s += a; }
    __device__ __forceinline__ double value() const { return s; }
};
template <>
struct SumAcc<float> {
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void add_pair(float p, float pe)
    {
        const float s = __fadd_rn(hi, p);   // two-sum: s + e = hi + p exactly
        const float bp = __fsub_rn(s, hi);
        const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(p, bp));
        const float l = __fadd_rn(lo, __fadd_rn(e, pe));
        hi = __fadd_rn(s, l);               // renormalise: |lo| <= half an ulp of hi
        lo = __fsub_rn(l, __fsub_rn(hi, s));
    }
    __device__ __forceinline__ void add_prod(float a, float b)
    {
        const float p = __fmul_rn(a, b);
        add_pair(p, __fmaf_rn(a, b, -p));
    }
    __device__ __forceinline__ void add(float a) { add_pair(a, 0.f); }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

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

// cell = floor(hi + lo) and frac = (hi + lo) - cell for an exact high part
// and a low part of a few cells at most, without forming hi + lo (whose
// rounding at |hi| ~ 1e3 would be ~1e-4).
__device__ __forceinline__ void split_floor(float hi, float lo, float& cell, float& frac)
{
    const float fl = floorf(hi);
    const float fr = __fadd_rn(__fsub_rn(hi, fl), lo);
    const float f2 = floorf(fr);
    cell = __fadd_rn(fl, f2);
    frac = __fsub_rn(fr, f2);
}

// Exact sample coordinate v = a*k1 + b*k2 + mid for integer-valued offsets
// k1, k2 and coefficients split as a = a_hi + a_lo, b = b_hi + b_lo (a_hi,
// b_hi multiples of 2^-q with q chosen on the host so that every partial sum
// of the high part fits in 24 bits).  The high part is then exact, the low
// part is below one cell, and the returned cell = floor(v) and frac = v -
// cell are correct to ~1e-7 (host tables: tables.cpp).  A value the high
// part cannot hold exactly lies outside the grid, before and after rounding.
__device__ __forceinline__ void exact_coord(float a_hi, float b_hi, float a_lo, float b_lo, float k1, float k2,
                                            float mid, float& cell, float& frac)
{
    split_floor(__fmaf_rn(a_hi, k1, __fmaf_rn(b_hi, k2, mid)), __fmaf_rn(a_lo, k1, __fmul_rn(b_lo, k2)), cell,
                frac);
}

// Sample coordinates along one projector ray (tomography/tv_hpc.F90:144-146):
//   xr = c*(jx-m) - s*dy + m,  yr = s*(jx-m) + c*dy + m,  dy = jy - m (+ off)
// at(dx) returns the cells x1 = floor(xr), y1 = floor(yr) and the bilinear
// weights wxl = x1+1-xr, wxh = xr-x1 (and the same in y).
// EX = false: the reference's operation order in Real (single or double).
// EX = true (single only): exact positions from the split FP64 tables.
template <typename Real, bool EX>
struct ProjRay {
    Real s, c, sdy, cdy, mid;
    __device__ ProjRay(const Real* sc, const float4*, int t, int jy, Real m, const Real* off_t) : mid(m)
    {
        s = sc[2 * t];
        c = sc[2 * t + 1];
        const Real dyv = off_t ? sub_rn(add_rn((Real)jy, *off_t), m) : (Real)jy - m;
        sdy = mul_rn(s, dyv);
        cdy = mul_rn(c, dyv);
    }
    __device__ __forceinline__ void at(Real dxv, int& x1, int& y1, Real& wxl, Real& wxh, Real& wyl, Real& wyh) const
    {
        const Real xr = add_rn(sub_rn(mul_rn(c, dxv), sdy), mid);
        const Real yr = add_rn(add_rn(mul_rn(s, dxv), cdy), mid);
        const Real x1f = rfloor(xr), y1f = rfloor(yr);
        x1 = (int)x1f;
        y1 = (int)y1f;
        wxl = add_rn(x1f, Real(1)) - xr;
        wxh = xr - x1f;
        wyl = add_rn(y1f, Real(1)) - yr;
        wyh = yr - y1f;
    }
};

template <>
struct ProjRay<float, true> {
    float sa, ca, sr, cr, bxh, byh, bxl, byl;
    __device__ ProjRay(const float*, const float4* xsc, int t, int jy, float m, const float* off_t)
    {
        const float4 x = __ldg(xsc + t);
        sa = x.x;
        ca = x.y;
        sr = x.z;
        cr = x.w;
        const float dy = (float)jy - m;
        bxh = __fmaf_rn(-sa, dy, m);   // exact (see exact_coord)
        byh = __fmaf_rn(ca, dy, m);
        bxl = __fmul_rn(-sr, dy);
        byl = __fmul_rn(cr, dy);
        if (off_t) {                   // a detector offset joins the low part
            const float o = *off_t;
            bxl = __fmaf_rn(-sa, o, __fmaf_rn(-sr, o, bxl));
            byl = __fmaf_rn(ca, o, __fmaf_rn(cr, o, byl));
        }
    }
    __device__ __forceinline__ void at(float dx, int& x1, int& y1, float& wxl, float& wxh, float& wyl,
                                       float& wyh) const
    {
        float cx, cy;
        split_floor(__fmaf_rn(ca, dx, bxh), __fmaf_rn(cr, dx, bxl), cx, wxh);
        split_floor(__fmaf_rn(sa, dx, byh), __fmaf_rn(sr, dx, byl), cy, wyh);
        x1 = (int)cx;
        y1 = (int)cy;
        wxl = __fsub_rn(1.f, wxh);
        wyl = __fsub_rn(1.f, wyh);
    }
};

// Paired single-precision FMA (sm_100 and later): d = a * b + c on both
// halves, each rounded as fmaf.
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c)
{
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tmov.b64 rc, {%6, %7};\n\t"
        "fma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}

// Steps jx of one ray (bin offset dy = jy - m) whose sample can lie in a
// valid cell, 2 <= xr < N and 2 <= yr < N, from the real-valued line
// (tomography/tv_hpc.F90:144-149) with a margin of two steps; a coordinate
// that hardly moves along the ray (|cos| or |sin| < 1e-3) is left
// unconstrained.  lo > hi: none.
__device__ __forceinline__ void valid_steps(float s, float c, float dy, float mid, int N, int& lo, int& hi)
{
    float a = -1e30f, b = 1e30f;   // bounds on jx - m
    auto axis = [&](float slope, float off) {
        if (fabsf(slope) < 1e-3f) return;
        const float t0 = (2.f - off) / slope, t1 = ((float)N - off) / slope;
        a = fmaxf(a, fminf(t0, t1));
        b = fminf(b, fmaxf(t0, t1));
    };
    axis(c, mid - s * dy);   // xr = c (jx - m) - s dy + m
    axis(s, mid + c * dy);   // yr = s (jx - m) + c dy + m
    lo = max(1, (int)floorf(fmaxf(a + mid, -1e8f)) - 2);
    hi = min(N, (int)ceilf(fminf(b + mid, 1e8f)) + 2);
}

// Lets kernel K use up to 227 KB of dynamic shared memory on the current
// device (the attribute is per device; set once per device, thread-safe).
template <auto K>
inline void max_dynamic_smem()
{
    static std::atomic<unsigned long long> done{0};
    int dev = 0;
    cudaGetDevice(&dev);
    const unsigned long long bit = 1ull << (dev & 63);
    if (done.load(std::memory_order_acquire) & bit) return;
    cudaFuncSetAttribute(K, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
    done.fetch_or(bit, std::memory_order_release);
}

}  // namespace acu
