// Projection preprocessing kernels: flat/dark averages and log-normalisation
// (tomography/fits_to_hpc.F90:183-244), the 0/180-degree pick
// (projections_to_sinogram_hpc.F90:141-224), rotation-axis registration
// (:231-364, plus a cross-correlation variant), the 27-point median (:426-452),
// the bilinear resample (:456-470) and the transpose to slice-major sinograms
// (:481-487).
//
// Arithmetic that decides an index or a comparison is written with explicit
// round-to-nearest operations so that it matches the single-precision
// reference operation for operation.
#include <algorithm>
#include <climits>
#include <cmath>

#include "../../include/acumen_gpu.h"
#include "common.cuh"
#include "prep.h"

namespace acu {

template <typename Tin>
__device__ __forceinline__ float to_f(Tin v) { return (float)v; }

// ---- frame averages (fits_to_hpc.F90:183-210): running sum in frame order ----
template <typename Tin>
__global__ void k_frame_average(int nframes, long npix, const Tin* __restrict__ frames, float* __restrict__ out)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < npix; i += (long)gridDim.x * blockDim.x) {
        float s = 0.0f;
        for (int j = 0; j < nframes; ++j) s = __fadd_rn(s, to_f(frames[(size_t)j * npix + i]));
        out[i] = __fdiv_rn(s, (float)nframes);
    }
}

// ---- log-normalisation (fits_to_hpc.F90:243 mode 0, :244 mode 1) ------------
template <typename Tin>
__global__ void k_normalize(int mode, long npix, long total, const Tin* __restrict__ raw, const float* __restrict__ ob,
                            const float* __restrict__ df, float* __restrict__ out)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const long k = i % npix;
        const float I = to_f(raw[i]);
        float v;
        if (mode == 0) {
            v = -logf(__fdiv_rn(I, fmaxf(ob[k], 1.0f)));
        } else {
            const float d = df[k];
            v = -logf(__fdiv_rn(fmaxf(__fsub_rn(I, d), 1e-16f), fmaxf(__fsub_rn(ob[k], d), 1.0f)));
        }
        out[i] = v;
    }
}

// Vectorised form for frames of a multiple of 8 pixels with 16-byte aligned
// arrays: one thread normalises 8 consecutive pixels of one projection (a
// 16-byte load of uint16 counts or two of floats, two 16-byte loads of each
// flat/dark average, two 16-byte stores); grid.y walks the projections, so no
// 64-bit division is needed.  Same arithmetic per pixel as k_normalize.
__device__ __forceinline__ void load8(const uint16_t* p, float (&v)[8])
{
    const uint4 u = __ldg(reinterpret_cast<const uint4*>(p));
    const unsigned w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        v[2 * i] = (float)(w[i] & 0xffffu);
        v[2 * i + 1] = (float)(w[i] >> 16);
    }
}
__device__ __forceinline__ void load8(const float* p, float (&v)[8])
{
    const float4 a = __ldg(reinterpret_cast<const float4*>(p)), b = __ldg(reinterpret_cast<const float4*>(p) + 1);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}

template <typename Tin>
__global__ void __launch_bounds__(256) k_normalize8(int mode, int nproj, long nvec, const Tin* __restrict__ raw,
                                                    const float* __restrict__ ob, const float* __restrict__ df,
                                                    float* __restrict__ out)
{
    for (int p = blockIdx.y; p < nproj; p += gridDim.y) {
        const Tin* rp = raw + (size_t)p * nvec * 8;
        float* op = out + (size_t)p * nvec * 8;
        for (long v = blockIdx.x * (long)blockDim.x + threadIdx.x; v < nvec; v += (long)gridDim.x * blockDim.x) {
            float I[8], o[8], d[8];
            load8(rp + v * 8, I);
            load8(ob + v * 8, o);
            if (mode == 0) {
#pragma unroll
                for (int i = 0; i < 8; ++i) I[i] = -logf(__fdiv_rn(I[i], fmaxf(o[i], 1.0f)));
            } else {
                load8(df + v * 8, d);
#pragma unroll
                for (int i = 0; i < 8; ++i)
                    I[i] = -logf(__fdiv_rn(fmaxf(__fsub_rn(I[i], d[i]), 1e-16f), fmaxf(__fsub_rn(o[i], d[i]), 1.0f)));
            }
            float4* q = reinterpret_cast<float4*>(op + v * 8);
            q[0] = make_float4(I[0], I[1], I[2], I[3]);
            q[1] = make_float4(I[4], I[5], I[6], I[7]);
        }
    }
}

// ---- lerp between two projections (projections_to_sinogram_hpc.F90:162) ------
__global__ void k_lerp(long n, const float* __restrict__ a, const float* __restrict__ b, float ta, float tb,
                       float target, float* __restrict__ out)
{
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        out[i] = __fadd_rn(__fdiv_rn(__fmul_rn(__fsub_rn(target, ta), __fsub_rn(b[i], a[i])), __fsub_rn(tb, ta)),
                           a[i]);
}

// ---- bilinear resample with the reference's clamps (:456-470) ---------------
struct ResampleGeom {
    int ndet, nrows, add;
    float cth, sth, shift;
};

__device__ __forceinline__ float resample_at(const ResampleGeom& g, const float* __restrict__ src, int jx, int jy)
{
    const float mx = __fdiv_rn((float)(g.ndet + g.add - 1), 2.0f);
    const float my = __fdiv_rn((float)(g.nrows - 1), 2.0f);
    const float ss = (float)g.ndet;
    const float ax = __fsub_rn(__fsub_rn((float)jx, mx), __fmul_rn(ss, g.shift));
    const float ay = __fsub_rn((float)jy, my);
    float xr = __fadd_rn(__fsub_rn(__fmul_rn(g.cth, ax), __fmul_rn(g.sth, ay)), mx);
    float yr = __fadd_rn(__fadd_rn(__fmul_rn(g.sth, ax), __fmul_rn(g.cth, ay)), my);
    xr = fminf(fmaxf(xr, 1.0f), (float)g.ndet);
    yr = fminf(fmaxf(yr, 1.0f), (float)g.nrows);
    int y1 = min(max((int)floorf(yr), 1), g.nrows);
    int y2 = min(max(y1 + 1, 1), g.nrows);
    int x1 = min(max((int)floorf(xr), 1), g.ndet);
    int x2 = min(max(x1 + 1, 1), g.ndet);
    const float wxl = __fsub_rn((float)x2, xr), wxh = __fsub_rn(xr, (float)x1);
    const float wyl = __fsub_rn((float)y2, yr), wyh = __fsub_rn(yr, (float)y1);
    const size_t r1 = (size_t)(y1 - 1) * g.ndet, r2 = (size_t)(y2 - 1) * g.ndet;
    float acc = __fmul_rn(__fmul_rn(src[r1 + x1 - 1], wxl), wyl);
    acc = __fadd_rn(acc, __fmul_rn(__fmul_rn(src[r1 + x2 - 1], wxh), wyl));
    acc = __fadd_rn(acc, __fmul_rn(__fmul_rn(src[r2 + x1 - 1], wxl), wyh));
    acc = __fadd_rn(acc, __fmul_rn(__fmul_rn(src[r2 + x2 - 1], wxh), wyh));
    return acc;
}

__global__ void k_resample(ResampleGeom g, const float* __restrict__ src, float* __restrict__ out)
{
    const int nx = g.ndet + g.add;
    const long n = (long)nx * g.nrows;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int jx = (int)(i % nx) + 1, jy = (int)(i / nx) + 1;
        out[i] = resample_at(g, src, jx, jy);
    }
}

// ---- registration objective (:279-284 / :308-313 / :346-351) ----------------
// sum |V0(jx,jy) - V180(nx-jx+1,jy)| over the padded grid: one FP64 partial
// per block, summed afterwards in block order (deterministic).
__global__ void __launch_bounds__(256) k_mirror_error(ResampleGeom g, const float* __restrict__ p0,
                                                      const float* __restrict__ p180, double* __restrict__ part)
{
    __shared__ double sh[32];
    const int nx = g.ndet + g.add;
    const long n = (long)nx * g.nrows;
    double acc = 0.0;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int jx = (int)(i % nx) + 1, jy = (int)(i / nx) + 1;
        const float a = resample_at(g, p0, jx, jy);
        const float b = resample_at(g, p180, nx - jx + 1, jy);
        acc += (double)fabsf(__fsub_rn(a, b));
    }
    const double r = block_sum(acc, sh);
    if (threadIdx.x == 0 && threadIdx.y == 0) part[blockIdx.x] = r;
}

// centre-of-mass sums (:234-243): tm, cmx_0, cmx_180 as FP64 partials
__global__ void __launch_bounds__(256) k_com(int ndet, int nrows, int add, const float* __restrict__ p0,
                                             const float* __restrict__ p180, double* __restrict__ part)
{
    __shared__ double sh[32];
    double tm = 0.0, c0 = 0.0, c1 = 0.0;
    const long n = (long)ndet * nrows;
    const float nda = (float)(ndet + add);
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int jx = (int)(i % ndet) + 1;
        const float a = p0[i], b = p180[i];
        const float w = __fsub_rn(__fsub_rn(__fdiv_rn(__fmul_rn(__fmul_rn(2.0f, nda), (float)(jx - 1)),
                                                      (float)(ndet + add - 1)),
                                            (float)ndet),
                                  (float)add);
        tm += (double)a + (double)b;
        c0 += (double)__fmul_rn(a, w);
        c1 += (double)__fmul_rn(b, w);
    }
    double r = block_sum(tm, sh);
    if (threadIdx.x == 0) part[3 * blockIdx.x] = r;
    r = block_sum(c0, sh);
    if (threadIdx.x == 0) part[3 * blockIdx.x + 1] = r;
    r = block_sum(c1, sh);
    if (threadIdx.x == 0) part[3 * blockIdx.x + 2] = r;
}

// fixed-order sum of `n` partials with stride `stride` (offset `off`) into out[0]
__global__ void k_sum_partials(const double* __restrict__ part, int n, int stride, int off, double* __restrict__ out)
{
    __shared__ double sh[32];
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) v += part[(size_t)i * stride + off];
    const double r = block_sum(v, sh);
    if (threadIdx.x == 0) out[0] = r;
}

// ---- cross-correlation registration (new) --------------------------------------
// C(k) = sum_{x,y} p0(x,y) * p180(ndet-1-x+k, y) with every product truncated
// to 2^-32 fixed point and summed exactly in 128-bit integers: integer sums do
// not depend on their order, so the argmax is bit-exact against the CPU oracle,
// and a 128-bit sum of n terms below 2^63 cannot wrap for n < 2^64.  A product
// that is not finite or not below 2^31 in magnitude (its fixed-point value would
// not fit 64 bits) sets the range flag and is left out; the host then rejects
// the input.  Every element of p0 and p180 meets a partner at k = 0, so every
// element is checked.
//
// Scratch layout (unsigned 64-bit words): lag i's sum at [2i] (low word) and
// [2i+1] (high word, two's complement), then one word holding the argmax
// index (low 32 bits) and the range flag (high 32 bits).
constexpr double kFixScale = 4294967296.0;     // 2^32
constexpr double kFixLimit = 2147483648.0;     // |product| < 2^31

// 128-bit atomic add from two 64-bit atomics: the low words add modulo 2^64
// and each addition that wraps carries one into the high word, so the pair
// holds the exact sum modulo 2^128 whatever the order of the additions.
__device__ __forceinline__ void atomic_add_i128(unsigned long long* w, __int128 v)
{
    const unsigned long long lo = (unsigned long long)v, hi = (unsigned long long)(v >> 64);
    const unsigned long long old = atomicAdd(w, lo);
    const unsigned long long carry = (old + lo < old) ? 1ull : 0ull;
    if (hi + carry) atomicAdd(w + 1, hi + carry);
}

__device__ __forceinline__ __int128 shfl_down_i128(__int128 v, int o)
{
    const unsigned long long lo = __shfl_down_sync(0xffffffffu, (unsigned long long)v, o);
    const long long hi = __shfl_down_sync(0xffffffffu, (long long)(v >> 64), o);
    return ((__int128)hi << 64) | (__int128)lo;
}

__global__ void __launch_bounds__(256) k_xcorr(int ndet, int nrows, int kmax, const float* __restrict__ p0,
                                               const float* __restrict__ p180, unsigned long long* __restrict__ w)
{
    const int k = (int)blockIdx.y - kmax;
    const long n = (long)ndet * nrows;
    __int128 acc = 0;
    bool bad = false;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int x = (int)(i % ndet), y = (int)(i / ndet);
        const int xm = ndet - 1 - x + k;
        if (xm >= 0 && xm < ndet) {
            const double p = (double)p0[i] * (double)p180[(size_t)y * ndet + xm];   // exact
            if (fabs(p) < kFixLimit) acc += (__int128)__double2ll_rd(p * kFixScale);
            else bad = true;                                                          // also NaN
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += shfl_down_i128(acc, o);
    if ((threadIdx.x & 31) == 0 && acc != 0) atomic_add_i128(&w[2 * blockIdx.y], acc);
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) {
        unsigned int* flag = reinterpret_cast<unsigned int*>(w + 2 * (2 * kmax + 1)) + 1;
        atomicOr(flag, 1u);
    }
}

__device__ __forceinline__ bool i128_better(long long ah, unsigned long long al, int ai, long long bh,
                                            unsigned long long bl, int bi)
{
    if (ah != bh) return ah > bh;
    if (al != bl) return al > bl;
    return ai < bi;
}

// Warp-shuffle argmax over the nk 128-bit correlation values (ties: lowest index).
__global__ void k_argmax(int nk, unsigned long long* __restrict__ w)
{
    long long bh = LLONG_MIN;
    unsigned long long bl = 0;
    int bi = 0x7fffffff;
    for (int i = threadIdx.x; i < nk; i += 32) {
        const long long h = (long long)w[2 * i + 1];
        const unsigned long long l = w[2 * i];
        if (i128_better(h, l, i, bh, bl, bi)) { bh = h; bl = l; bi = i; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const long long oh = __shfl_down_sync(0xffffffffu, bh, o);
        const unsigned long long ol = __shfl_down_sync(0xffffffffu, bl, o);
        const int oi = __shfl_down_sync(0xffffffffu, bi, o);
        if (i128_better(oh, ol, oi, bh, bl, bi)) { bh = oh; bl = ol; bi = oi; }
    }
    if (threadIdx.x == 0) reinterpret_cast<int*>(w + 2 * nk)[0] = bi;
}

// ---- 27-point median (:426-452): the reference's descending exchange sort,
// passes 1..14 (the later passes do not touch element 14), with the
// intended slots 1..27 ------------------------------------------------------------
// When the 27 values hold no NaN and no zero, every selection of the 14th
// largest returns the same bits (equal finite non-zero floats, and equal
// infinities, are bitwise equal), so a cheaper selection is used: forgetful
// selection, which keeps 15 candidates, moves their minimum and maximum to the
// ends with compare-exchanges (min/max pairs), drops both, takes in the next
// value and repeats -- 390 min/max operations instead of the 273
// compare-and-swap steps (819 instructions) of the exchange sort.  With a NaN
// (whose comparisons are false) or a signed zero present, the exchange sort
// itself decides, bit for bit.
__device__ __forceinline__ void cx_minmax(float& a, float& b)
{
    const float lo = fminf(a, b), hi = fmaxf(a, b);
    a = lo;
    b = hi;
}

__device__ __forceinline__ float median27_select(float (&r)[27])
{
    bool plain = true;
#pragma unroll
    for (int i = 0; i < 27; ++i) plain &= fabsf(r[i]) > 0.0f;   // false for NaN and +-0
    if (plain) {
#pragma unroll
        for (int A = 0; A <= 12; ++A) {
#pragma unroll
            for (int i = A + 1; i <= 14; ++i) cx_minmax(r[A], r[i]);   // minimum of r[A..14] to r[A]
#pragma unroll
            for (int i = A + 1; i < 14; ++i) cx_minmax(r[i], r[14]);   // maximum to r[14]
            if (A < 12) r[14] = r[15 + A];                               // drop both, take the next
        }
        return r[13];
    }
#pragma unroll
    for (int a = 0; a < 14; ++a) {
        float ra = r[a];
#pragma unroll
        for (int b = a + 1; b < 27; ++b) {
            const float rb = r[b];
            const bool sw = rb > ra;
            r[b] = sw ? ra : rb;
            ra = sw ? rb : ra;
        }
        r[a] = ra;
    }
    return r[13];
}

// The median at (jx, jy) (1-based) of the 3x3 neighbourhood, clamped to the
// frame, in the previous (dl), current (dc) and next (dr) projection.
__device__ __forceinline__ float median27_at(const float* __restrict__ dl, const float* __restrict__ dc,
                                             const float* __restrict__ dr, int ndet, int nrows, int jx, int jy)
{
    float r[27];
#pragma unroll
    for (int jxs = -1; jxs <= 1; ++jxs)
#pragma unroll
        for (int jys = -1; jys <= 1; ++jys) {
            const int cx = min(max(jx + jxs, 1), ndet), cy = min(max(jy + jys, 1), nrows);
            const size_t o = (size_t)(cy - 1) * ndet + (cx - 1);
            const int slot = 3 * (jxs + 1) + (jys + 1);
            r[slot] = __ldg(dl + o);
            r[slot + 9] = __ldg(dc + o);
            r[slot + 18] = __ldg(dr + o);
        }
    return median27_select(r);
}

__global__ void __launch_bounds__(128) k_median27(int ndet, int nrows, int nproj_chunk, int p_first, int nfiles,
                                                  const float* __restrict__ proj, float* __restrict__ out)
{
    const long npix = (long)ndet * nrows;
    const long total = npix * nproj_chunk;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int pc = (int)(i / npix);
        const long k = i % npix;
        const int p = p_first + pc;
        const int jx = (int)(k % ndet) + 1, jy = (int)(k / ndet) + 1;
        const float* dc = proj + (size_t)p * npix;
        const float* dl = p > 0 ? dc - npix : dc;
        const float* dr = p < nfiles - 1 ? dc + npix : dc;
        out[(size_t)pc * npix + k] = median27_at(dl, dc, dr, ndet, nrows, jx, jy);
    }
}

// resample + transpose of a chunk of projections into the slice-major
// sinograms sino[row][projection][det] (:456-487)
__global__ void k_resample_to_sino(ResampleGeom g, int nproj_chunk, int p_first, int nfiles,
                                   const float* __restrict__ med, float* __restrict__ sino)
{
    const int nx = g.ndet + g.add;
    const long per = (long)nx * g.nrows;
    const long total = per * nproj_chunk;
    const long npix = (long)g.ndet * g.nrows;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const int pc = (int)(i / per);
        const long k = i % per;
        const int jx = (int)(k % nx) + 1, jy = (int)(k / nx) + 1;
        const float v = resample_at(g, med + (size_t)pc * npix, jx, jy);
        sino[((size_t)(jy - 1) * nfiles + (p_first + pc)) * nx + (jx - 1)] = v;
    }
}

// ---- launchers -----------------------------------------------------------------
static inline unsigned nblocks(long n, int threads, unsigned cap = 8192)
{
    long b = (n + threads - 1) / threads;
    return (unsigned)(b < (long)cap ? (b < 1 ? 1 : b) : cap);
}

void launch_frame_average_u16(int nf, long npix, const uint16_t* f, float* out, cudaStream_t st)
{
    k_frame_average<uint16_t><<<nblocks(npix, 256), 256, 0, st>>>(nf, npix, f, out);
}
void launch_frame_average_f32(int nf, long npix, const float* f, float* out, cudaStream_t st)
{
    k_frame_average<float><<<nblocks(npix, 256), 256, 0, st>>>(nf, npix, f, out);
}
static bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

template <typename Tin>
static void launch_normalize(int mode, int nproj, long npix, const Tin* raw, const float* ob, const float* df,
                             float* out, cudaStream_t st)
{
    if (npix % 8 == 0 && aligned16(raw) && aligned16(ob) && aligned16(out) && (mode == 0 || aligned16(df))) {
        const long nvec = npix / 8;
        dim3 grd(nblocks(nvec, 256, 2048), (unsigned)std::min(nproj, 32768));
        k_normalize8<Tin><<<grd, 256, 0, st>>>(mode, nproj, nvec, raw, ob, df, out);
    } else {
        const long total = npix * nproj;
        k_normalize<Tin><<<nblocks(total, 256), 256, 0, st>>>(mode, npix, total, raw, ob, df, out);
    }
}
void launch_normalize_u16(int mode, int nproj, long npix, const uint16_t* raw, const float* ob, const float* df,
                          float* out, cudaStream_t st)
{
    launch_normalize<uint16_t>(mode, nproj, npix, raw, ob, df, out, st);
}
void launch_normalize_f32(int mode, int nproj, long npix, const float* raw, const float* ob, const float* df,
                          float* out, cudaStream_t st)
{
    launch_normalize<float>(mode, nproj, npix, raw, ob, df, out, st);
}
void launch_lerp(long n, const float* a, const float* b, float ta, float tb, float target, float* out,
                 cudaStream_t st)
{
    k_lerp<<<nblocks(n, 256), 256, 0, st>>>(n, a, b, ta, tb, target, out);
}
void launch_resample(int ndet, int nrows, const float* src, float cth, float sth, float shift, float* out,
                     cudaStream_t st)
{
    ResampleGeom g{ndet, nrows, ndet % 2 == 0 ? 1 : 0, cth, sth, shift};
    k_resample<<<nblocks((long)(ndet + g.add) * nrows, 256), 256, 0, st>>>(g, src, out);
}
int mirror_error_blocks(int ndet, int nrows)
{
    return (int)nblocks((long)(ndet + 1) * nrows, 256, 1024);
}
void launch_mirror_error(int ndet, int nrows, const float* p0, const float* p180, float cth, float sth, float shift,
                         double* part, int nblk, double* out, cudaStream_t st)
{
    ResampleGeom g{ndet, nrows, ndet % 2 == 0 ? 1 : 0, cth, sth, shift};
    k_mirror_error<<<nblk, 256, 0, st>>>(g, p0, p180, part);
    k_sum_partials<<<1, 256, 0, st>>>(part, nblk, 1, 0, out);
}
void launch_com(int ndet, int nrows, const float* p0, const float* p180, double* part, int nblk, double* out3,
                cudaStream_t st)
{
    k_com<<<nblk, 256, 0, st>>>(ndet, nrows, ndet % 2 == 0 ? 1 : 0, p0, p180, part);
    for (int j = 0; j < 3; ++j) k_sum_partials<<<1, 256, 0, st>>>(part, nblk, 3, j, out3 + j);
}
size_t xcorr_scratch_words(int kmax) { return 2 * (size_t)(2 * kmax + 1) + 1; }

namespace {
template <typename T>
struct same_t {
    using type = T;
};
// cudaLaunchKernel with typed arguments: returns this launch's own error and
// leaves earlier, unrelated errors of the caller pending.
template <typename... P>
cudaError_t launch_k(void (*k)(P...), dim3 grd, dim3 blk, cudaStream_t st, typename same_t<P>::type... args)
{
    void* a[] = {&args...};
    return cudaLaunchKernel(reinterpret_cast<const void*>(k), grd, blk, a, 0, st);
}
}  // namespace

cudaError_t launch_xcorr(int ndet, int nrows, int kmax, const float* p0, const float* p180,
                         unsigned long long* scratch, cudaStream_t st)
{
    const int nk = 2 * kmax + 1;
    cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(unsigned long long) * xcorr_scratch_words(kmax), st);
    if (e != cudaSuccess) return e;
    dim3 grd(nblocks((long)ndet * nrows, 256, 64), nk);
    e = launch_k(k_xcorr, grd, dim3(256), st, ndet, nrows, kmax, p0, p180, scratch);
    if (e != cudaSuccess) return e;
    return launch_k(k_argmax, dim3(1), dim3(32), st, nk, scratch);
}

int xcorr_finish(int kmax, const unsigned long long* h, int64_t* corr_out, int* k_best, double* k_sub,
                 const char** why)
{
    const int nk = 2 * kmax + 1;
    const int bi = (int)(unsigned int)(h[2 * nk] & 0xffffffffu);
    const unsigned int flag = (unsigned int)(h[2 * nk] >> 32);
    if (flag) {
        *why = "a projection holds a value that is not finite, or a product p0*p180 of magnitude >= 2^31";
        return ACU_ERR_INVALID;
    }
    if (bi < 0 || bi >= nk) {
        *why = "the correlation argmax is out of range";
        return ACU_ERR_CUDA;
    }
    auto fits = [&](int i) {
        const long long hi = (long long)h[2 * i + 1];
        const long long lo = (long long)h[2 * i];
        return hi == (lo < 0 ? -1ll : 0ll);
    };
    auto to_double = [&](int i) {   // the sum as a double (exact conversion of an int64 when it fits)
        if (fits(i)) return (double)(long long)h[2 * i];
        return ldexp((double)(long long)h[2 * i + 1], 64) + (double)h[2 * i];
    };
    if (corr_out) {
        for (int i = 0; i < nk; ++i)
            if (!fits(i)) {
                *why = "a correlation sum exceeds the int64 range of corr_out (pass corr_out = NULL for the lag "
                       "alone)";
                return ACU_ERR_UNSUPPORTED;
            }
        for (int i = 0; i < nk; ++i) corr_out[i] = (int64_t)(long long)h[2 * i];
    }
    double frac = 0.0;
    if (bi > 0 && bi < nk - 1) {
        const double cm = to_double(bi - 1), c0 = to_double(bi), cp = to_double(bi + 1);
        const double den = cm - 2.0 * c0 + cp;
        if (den < 0.0) frac = 0.5 * (cm - cp) / den;
    }
    *k_best = bi - kmax;
    *k_sub = (double)(bi - kmax) + frac;
    return ACU_OK;
}
void launch_median27(int ndet, int nrows, int nchunk, int p_first, int nfiles, const float* proj, float* out,
                     cudaStream_t st)
{
    k_median27<<<nblocks((long)ndet * nrows * nchunk, 128, 65535), 128, 0, st>>>(ndet, nrows, nchunk, p_first,
                                                                                nfiles, proj, out);
}
void launch_resample_to_sino(int ndet, int nrows, int nchunk, int p_first, int nfiles, const float* med,
                             float cth, float sth, float shift, float* sino, cudaStream_t st)
{
    ResampleGeom g{ndet, nrows, ndet % 2 == 0 ? 1 : 0, cth, sth, shift};
    k_resample_to_sino<<<nblocks((long)(ndet + g.add) * nrows * nchunk, 256, 65535), 256, 0, st>>>(
        g, nchunk, p_first, nfiles, med, sino);
}

}  // namespace acu
