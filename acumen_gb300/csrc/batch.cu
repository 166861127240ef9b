// Ragged batches: many independent problems of different grid size N and
// angle count T (each one slice) solved together.  The projector and the
// backprojection are persistent kernels: every resident warp (projector) or
// block (backprojection) takes (problem, angle, 32-bin block) or (problem,
// pixel tile) items from a device counter until the list is exhausted, so one
// launch covers the whole batch with dynamic load balance; items are listed
// largest problem first.  The filter and the element-wise TV steps map one
// block per item.  The arithmetic is that of the uniform kernels
// (kernels_radon.cu, kernels_tv.cu), applied with each problem's geometry.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

#include "batch.h"
#include "common.cuh"
#include "ctx.h"
#include "tables.h"

namespace acu {

// One staggered ray of the single-slice projector (as radon_stag_ray<1> in
// kernels_radon.cu), through the image (TR = false) or its transpose, over the
// warp's steps i0..i1.
template <bool EX, bool TR>
__device__ __forceinline__ void radon_stag_ray_v1(const float* __restrict__ base, int N, int kb, int i0, int i1,
                                                  const ProjRay<float, EX>& ray, float mid, int jy,
                                                  float (&acc)[1])
{
    constexpr bool transposed = TR;
    for (int i = i0; i <= i1; ++i) {
        const int jx = i - kb;
        if (jx < 1 || jx > N || jy > N) continue;
        int x1, y1;
        float wxl, wxh, wyl, wyh;
        ray.at((float)jx - mid, x1, y1, wxl, wxh, wyl, wyh);
        if (min(x1, y1) > 1 && max(x1, y1) < N) {
            const float w11 = wxl * wyl, w21 = wxh * wyl, w12 = wxl * wyh, w22 = wxh * wyh;
            const int r0 = transposed ? x1 : y1, c0 = transposed ? y1 : x1;
            const float* q = base + (size_t)(r0 - 1) * N + (c0 - 1);
            const float wb = transposed ? w12 : w21, wc = transposed ? w21 : w12;
            acc[0] = fmaf(__ldg(q + N + 1), w22, fmaf(__ldg(q + N), wc, fmaf(__ldg(q + 1), wb, fmaf(__ldg(q), w11, acc[0]))));
        }
    }
}

// problem of item `it` in a list whose per-problem first items are field F
template <long long ProbDesc::*F>
__device__ __forceinline__ int find_prob(const ProbDesc* __restrict__ pd, int nprob, long long it)
{
    int lo = 0, hi = nprob - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pd[mid].*F <= it)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// ---- projector: one warp item = 32 rays of one angle of one problem --------
// Staggered rays through the image or its transpose (whichever the warp's
// rays spread along), as the uniform projector.
template <bool EX>
__global__ void __launch_bounds__(512) k_batch_radon(const ProbDesc* __restrict__ pd, int nprob,
                                                     const float* __restrict__ img, const float* __restrict__ IT,
                                                     float* __restrict__ sino, const float* __restrict__ sc,
                                                     const float4* __restrict__ xsc, long long total, int* counter)
{
    const int lane = threadIdx.x & 31;
    for (;;) {
        int it = 0;
        if (lane == 0) it = atomicAdd(counter, 1);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= total) break;
        const int p = find_prob<&ProbDesc::it_radon>(pd, nprob, it);
        const ProbDesc d = pd[p];
        const int local = (int)(it - d.it_radon);
        const int t = local / d.nbx, b = local % d.nbx;
        const int jy = b * 32 + lane + 1;
        const int N = d.N;
        const float s = sc[d.sc + 2 * t], c = sc[d.sc + 2 * t + 1];
        const ProjRay<float, EX> ray(sc + d.sc, xsc + d.sc / 2, t, jy, d.mid, nullptr);
        const bool transposed = fabsf(c) > fabsf(s);
        const float ratio = transposed ? -s / c : c / s;
        const int kb = __float2int_rn((float)lane * ratio);
        const int kend = __float2int_rn(31.f * ratio);
        // the warp's steps: those that can meet a valid cell (see valid_steps)
        int lo, hi;
        valid_steps(s, c, (float)jy - d.mid, d.mid, N, lo, hi);
        if (jy > N || lo > hi) {
            lo = 0x3fffffff;
            hi = -0x3fffffff;
        }
        const int i0 = max(1 + min(0, kend), __reduce_min_sync(0xffffffffu, lo + kb));
        const int i1 = min(N + max(0, kend), __reduce_max_sync(0xffffffffu, hi + kb));
        float acc[1] = {0.f};
        if (transposed)
            radon_stag_ray_v1<EX, true>(IT + d.img, N, kb, i0, i1, ray, d.mid, jy, acc);
        else
            radon_stag_ray_v1<EX, false>(img + d.img, N, kb, i0, i1, ray, d.mid, jy, acc);
        if (jy <= N) sino[d.sino + (size_t)t * N + (jy - 1)] = acc[0] / (float)N;
    }
}

// transposed copies of every problem's image, one block per 32 x 32 tile
__global__ void __launch_bounds__(256) k_batch_transpose(const ProbDesc* __restrict__ pd, int nprob,
                                                         const float* __restrict__ img, float* __restrict__ IT)
{
    __shared__ float tile[32][33];
    const long long it = blockIdx.x;
    const int p = find_prob<&ProbDesc::it_tr>(pd, nprob, it);
    const ProbDesc d = pd[p];
    const int N = d.N, nt = (N + 31) / 32;
    const int local = (int)(it - d.it_tr);
    const int x0 = (local % nt) * 32, y0 = (local / nt) * 32;
    const float* src = img + d.img;
    float* dst = IT + d.img;
    for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) {
        const int ty = i / 32, tx = i % 32;
        if (x0 + tx < N && y0 + ty < N) tile[ty][tx] = src[(size_t)(y0 + ty) * N + x0 + tx];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) {
        const int ty = i / 32, tx = i % 32;
        if (x0 + ty < N && y0 + tx < N) dst[(size_t)(x0 + ty) * N + y0 + tx] = tile[tx][ty];
    }
}

// ---- backprojection: one block item = a 32 x R pixel tile of one problem ----
template <bool EX>
__global__ void __launch_bounds__(512) k_batch_backproject(const ProbDesc* __restrict__ pd, int nprob,
                                                           const float* __restrict__ q, float* __restrict__ img,
                                                           const float* __restrict__ sc,
                                                           const float4* __restrict__ xsc,
                                                           const float* __restrict__ cmask, long long total,
                                                           int* counter)
{
    __shared__ int s_it;
    const int R = blockDim.y;
    for (;;) {
        if (threadIdx.x == 0 && threadIdx.y == 0) s_it = atomicAdd(counter, 1);
        __syncthreads();
        const int it = s_it;
        __syncthreads();
        if (it >= total) break;
        const int p = find_prob<&ProbDesc::it_bp>(pd, nprob, it);
        const ProbDesc d = pd[p];
        const int N = d.N;
        const int ntx = (N + 31) / 32;
        const int local = (int)(it - d.it_bp);
        const int jx = (local % ntx) * 32 + threadIdx.x + 1;
        const int jy = (local / ntx) * R + threadIdx.y + 1;
        if (jx > N || jy > N) continue;
        const size_t pix = (size_t)(jy - 1) * N + (jx - 1);
        const float cm = cmask[d.cm + pix];
        float acc = 0.f;
        if (cm != 0.f) {
            const float mid = d.mid;
            const float dx = (float)jx - mid, dy = (float)jy - mid;
            const float* qq = q + d.sino;
            const float* sct = sc + d.sc;
            const float4* xst = xsc + d.sc / 2;
            for (int t = 0; t < d.T; ++t) {
                float y1f, wl, wh;
                if constexpr (EX) {
                    const float4 x = __ldg(xst + t);
                    exact_coord(x.x, x.y, x.z, x.w, dx, dy, mid, y1f, wh);
                    wl = 1.f - wh;
                } else {
                    const float s = sct[2 * t], c = sct[2 * t + 1];
                    const float yr = add_rn(add_rn(mul_rn(s, dx), mul_rn(c, dy)), mid);
                    y1f = floorf(yr);
                    wl = add_rn(y1f, 1.f) - yr;
                    wh = yr - y1f;
                }
                const int y1 = (int)y1f;
                if (y1 > 1 && y1 < N) {
                    const float* row = qq + (size_t)t * N + (y1 - 1);
                    acc = fmaf(__ldg(row + 1), wh, fmaf(__ldg(row), wl, acc));
                }
            }
        }
        img[d.img + pix] = cm * acc;
    }
}

// ---- FFT filter: one block per (problem, pair of angles) -----------------------
__device__ float2* fft_ragged(float2* d0, float2* d1, const float2* __restrict__ tw, int twstep, int L)
{
    for (int Ns = 1; Ns < L;) {
        const int Rdx = ((L / Ns) % 4 == 0) ? 4 : 2;
        const int stride = (L / (Ns * Rdx)) * twstep;
        const int nb = L / Rdx;
        for (int j = threadIdx.x; j < nb; j += blockDim.x) {
            const int k = j % Ns;
            const int idxD = (j / Ns) * Ns * Rdx + k;
            auto cmul = [](float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); };
            if (Rdx == 4) {
                const float2 v0 = d0[j];
                const float2 v1 = cmul(d0[j + nb], tw[k * stride]);
                const float2 v2 = cmul(d0[j + 2 * nb], tw[2 * k * stride]);
                const float2 v3 = cmul(d0[j + 3 * nb], tw[3 * k * stride]);
                const float2 a = make_float2(v0.x + v2.x, v0.y + v2.y), bb = make_float2(v0.x - v2.x, v0.y - v2.y);
                const float2 c = make_float2(v1.x + v3.x, v1.y + v3.y), e = make_float2(v1.x - v3.x, v1.y - v3.y);
                const float2 dd = make_float2(e.y, -e.x);
                d1[idxD] = make_float2(a.x + c.x, a.y + c.y);
                d1[idxD + Ns] = make_float2(bb.x + dd.x, bb.y + dd.y);
                d1[idxD + 2 * Ns] = make_float2(a.x - c.x, a.y - c.y);
                d1[idxD + 3 * Ns] = make_float2(bb.x - dd.x, bb.y - dd.y);
            } else {
                const float2 v0 = d0[j];
                const float2 v1 = cmul(d0[j + nb], tw[k * stride]);
                d1[idxD] = make_float2(v0.x + v1.x, v0.y + v1.y);
                d1[idxD + Ns] = make_float2(v0.x - v1.x, v0.y - v1.y);
            }
        }
        __syncthreads();
        float2* t = d0;
        d0 = d1;
        d1 = t;
        Ns *= Rdx;
    }
    return d0;
}

__global__ void __launch_bounds__(256) k_batch_filter(const ProbDesc* __restrict__ pd, int nprob,
                                                      const float* __restrict__ sino, float* __restrict__ out,
                                                      const float* __restrict__ H, const float2* __restrict__ tw,
                                                      int Lmax)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const long long it = blockIdx.x;
    const int p = find_prob<&ProbDesc::it_fft>(pd, nprob, it);
    const ProbDesc d = pd[p];
    const int N = d.N, L = d.L;
    float2* d0 = reinterpret_cast<float2*>(smem_raw);
    float2* d1 = d0 + L;
    const int t0 = 2 * (int)(it - d.it_fft);
    const bool has_b = t0 + 1 < d.T;
    const float* a = sino + d.sino + (size_t)t0 * N;
    for (int n = threadIdx.x; n < L; n += blockDim.x)
        d0[n] = make_float2(n < N ? a[n] : 0.f, (n < N && has_b) ? a[N + n] : 0.f);
    __syncthreads();
    float2* res = fft_ragged(d0, d1, tw, Lmax / L, L);
    float2* other = res == d0 ? d1 : d0;
    const float* h = H + d.fh;
    for (int m = threadIdx.x; m < L; m += blockDim.x) {
        const float2 z = res[m];
        res[m] = make_float2(h[m] * z.x, -h[m] * z.y);
    }
    __syncthreads();
    float2* y = fft_ragged(res, other, tw, Lmax / L, L);
    float* o = out + d.sino + (size_t)t0 * N;
    for (int n = threadIdx.x; n < N; n += blockDim.x) {
        o[n] = y[n].x;
        if (has_b) o[N + n] = -y[n].y;
    }
}

// ---- element-wise: one block of 256 threads per 1024 pixels of one problem ----
constexpr int EWB = 1024;

struct EwSpan {
    const ProbDesc* d;
    size_t lo, hi;
};

__device__ __forceinline__ ProbDesc ew_desc(const ProbDesc* pd, int nprob, size_t& lo, size_t& hi)
{
    const long long it = blockIdx.x;
    const int p = find_prob<&ProbDesc::it_ew>(pd, nprob, it);
    const ProbDesc d = pd[p];
    lo = (size_t)(it - d.it_ew) * EWB;
    hi = min(lo + EWB, (size_t)d.N * d.N);
    return d;
}

__device__ __forceinline__ void ew_partial(double v, double* part)
{
    __shared__ double sh[32];
    const double r = block_sum(v, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = r;
}

__device__ __forceinline__ int wnext(int j, int N) { return j + 1 == N ? 0 : j + 1; }
__device__ __forceinline__ int wprev(int j, int N) { return j == 0 ? N - 1 : j - 1; }

__device__ __forceinline__ float lap5(const float* u, int N, int x, int y)
{
    const float c = u[(size_t)y * N + x];
    return (((4.f * c - u[(size_t)y * N + wprev(x, N)]) - u[(size_t)y * N + wnext(x, N)]) -
            u[(size_t)wprev(y, N) * N + x]) -
           u[(size_t)wnext(y, N) * N + x];
}

__global__ void k_batch_rhs(const ProbDesc* pd, int nprob, float mu, float lambda, const float* ifkt, const float* dx,
                            const float* bx, const float* dy, const float* by, float* rhs)
{
    size_t lo, hi;
    const ProbDesc d = ew_desc(pd, nprob, lo, hi);
    const int N = d.N;
    const size_t o = d.img;
    for (size_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const int x = (int)(i % N), y = (int)(i / N);
        const size_t ixn = o + (size_t)y * N + wnext(x, N), iyn = o + (size_t)wnext(y, N) * N + x, ii = o + i;
        float acc = dx[ixn] - bx[ixn];
        acc = acc - dx[ii];
        acc = acc + bx[ii];
        acc = acc + dy[iyn];
        acc = acc - by[iyn];
        acc = acc - dy[ii];
        acc = acc + by[ii];
        rhs[ii] = mu * ifkt[ii] + lambda * acc;
    }
}

__global__ void k_batch_resid(const ProbDesc* pd, int nprob, float mu, float lambda, const float* rhs,
                              const float* iukt, const float* uk, float* r, float* p, double* part)
{
    size_t lo, hi;
    const ProbDesc d = ew_desc(pd, nprob, lo, hi);
    const int N = d.N;
    const float* u = uk + d.img;
    SumAcc<float> acc;
    for (size_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const int x = (int)(i % N), y = (int)(i / N);
        const size_t ii = d.img + i;
        // iukt == nullptr: rhs already holds mu * iradon(fk - radon(uk))
        const float v = (rhs[ii] - mu * (iukt ? iukt[ii] : 0.f)) - lambda * lap5(u, N, x, y);
        r[ii] = v;
        p[ii] = v;
        acc.add_prod(v, v);
    }
    ew_partial(acc.value(), part);
}

__global__ void k_batch_apply(const ProbDesc* pd, int nprob, float mu, float lambda, const float* irpt,
                              const float* p, float* Ap, double* part)
{
    size_t lo, hi;
    const ProbDesc d = ew_desc(pd, nprob, lo, hi);
    const int N = d.N;
    const float* pp = p + d.img;
    SumAcc<float> acc;
    for (size_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const int x = (int)(i % N), y = (int)(i / N);
        const size_t ii = d.img + i;
        const float v = mu * irpt[ii] + lambda * lap5(pp, N, x, y);
        Ap[ii] = v;
        acc.add_prod(pp[i], v);
    }
    ew_partial(acc.value(), part);
}

__global__ void k_batch_update(const ProbDesc* pd, int nprob, const float* p, const float* Ap, float* uk, float* r,
                               const double* alpha, double* part)
{
    size_t lo, hi;
    const ProbDesc d = ew_desc(pd, nprob, lo, hi);
    const float al = (float)alpha[find_prob<&ProbDesc::it_ew>(pd, nprob, blockIdx.x)];
    SumAcc<float> acc;
    for (size_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const size_t ii = d.img + i;
        uk[ii] = uk[ii] + al * p[ii];
        const float v = r[ii] - al * Ap[ii];
        r[ii] = v;
        acc.add_prod(v, v);
    }
    ew_partial(acc.value(), part);
}

__global__ void k_batch_pupdate(const ProbDesc* pd, int nprob, const float* r, float* p, const double* beta)
{
    size_t lo, hi;
    const ProbDesc d = ew_desc(pd, nprob, lo, hi);
    const float be = (float)beta[find_prob<&ProbDesc::it_ew>(pd, nprob, blockIdx.x)];
    for (size_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const size_t ii = d.img + i;
        p[ii] = r[ii] + be * p[ii];
    }
}

__device__ __forceinline__ float shrink1(float t, float thr)
{
    if (t == 0.f) return 0.f;
    const float a = fabsf(t);
    return (fmaxf(a - thr, 0.f) * t) / a;
}

__global__ void k_batch_shrink(const ProbDesc* pd, int nprob, float lambda, const float* uk, float* dx, float* bx,
                               float* dy, float* by)
{
    size_t lo, hi;
    const ProbDesc d = ew_desc(pd, nprob, lo, hi);
    const int N = d.N;
    const float* u = uk + d.img;
    const float thr = 1.f / lambda;
    for (size_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const int x = (int)(i % N), y = (int)(i / N);
        const size_t ii = d.img + i;
        float t = (u[(size_t)y * N + wprev(x, N)] - u[i]) + bx[ii];
        const float ox = shrink1(t, thr);
        dx[ii] = ox;
        bx[ii] = t - ox;
        t = (by[ii] + u[(size_t)wprev(y, N) * N + x]) - u[i];
        const float oy = shrink1(t, thr);
        dy[ii] = oy;
        by[ii] = t - oy;
    }
}

__global__ void k_batch_fk(long long n, float* fk, const float* f, const float* ruk)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        fk[i] = (fk[i] + f[i]) - ruk[i];
}

__global__ void k_batch_diff(long long n, const float* a, const float* b, float* out)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = a[i] - b[i];
}

// ruk += alpha radon(p) over each problem's sinogram (blockIdx.y = problem)
__global__ void k_batch_sino_axpy(const ProbDesc* pd, const double* alpha, const float* x, float* y)
{
    const ProbDesc d = pd[blockIdx.y];
    const float al = (float)alpha[blockIdx.y];
    const long long n = (long long)d.T * d.N;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        y[d.sino + i] = y[d.sino + i] + al * x[d.sino + i];
}

__global__ void k_batch_finalize(const ProbDesc* pd, int nprob, long long n_ew, int which, const double* part,
                                 double* rsold, double* alpha, double* beta)
{
    __shared__ double sh[32];
    const int p = blockIdx.x;
    const long long lo = pd[p].it_ew, hi = p + 1 < nprob ? pd[p + 1].it_ew : n_ew;
    double v = 0.0;
    for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) v += part[i];
    const double sum = block_sum(v, sh);
    if (threadIdx.x == 0) {
        if (which == 0) rsold[p] = sum;
        else if (which == 1) alpha[p] = sum != 0.0 ? rsold[p] / sum : 0.0;
        else {
            beta[p] = rsold[p] != 0.0 ? sum / rsold[p] : 0.0;
            rsold[p] = sum;
        }
    }
}

// ---- launchers ---------------------------------------------------------------
static int sm_count()
{
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);   // a cached attribute query
    return n > 0 ? n : 1;
}

void batch_radon(const BatchDev& b, const float* img, float* sino, int slot, cudaStream_t st)
{
    k_batch_transpose<<<(unsigned)b.n_tr, 256, 0, st>>>(b.pd, b.nprob, img, b.IT);
    cudaMemsetAsync(b.counter + slot, 0, sizeof(int), st);
    const int threads = 32 * b.radon_warps;
    const int blocks = sm_count() * (2048 / threads);
    if (b.exact)
        k_batch_radon<true><<<blocks, threads, 0, st>>>(b.pd, b.nprob, img, b.IT, sino, b.sc_fp, b.xsc_fp, b.n_radon,
                                                        b.counter + slot);
    else
        k_batch_radon<false><<<blocks, threads, 0, st>>>(b.pd, b.nprob, img, b.IT, sino, b.sc_fp, b.xsc_fp, b.n_radon,
                                                         b.counter + slot);
}
void batch_backproject(const BatchDev& b, const float* q, float* img, int slot, cudaStream_t st)
{
    cudaMemsetAsync(b.counter + slot, 0, sizeof(int), st);
    dim3 blk(32, b.bp_rows);
    const int blocks = sm_count() * (2048 / (32 * b.bp_rows));
    if (b.exact)
        k_batch_backproject<true><<<blocks, blk, 0, st>>>(b.pd, b.nprob, q, img, b.sc_bp, b.xsc_bp, b.cmask, b.n_bp,
                                                          b.counter + slot);
    else
        k_batch_backproject<false><<<blocks, blk, 0, st>>>(b.pd, b.nprob, q, img, b.sc_bp, b.xsc_bp, b.cmask, b.n_bp,
                                                           b.counter + slot);
}
void batch_filter(const BatchDev& b, const float* sino, float* out, cudaStream_t st)
{
    max_dynamic_smem<k_batch_filter>();
    const float* H = (b.exact && b.fft_h_x) ? b.fft_h_x : b.fft_h;   // exact positions: FP64 taps
    k_batch_filter<<<(unsigned)b.n_fft, 256, 2 * (size_t)b.Lmax * sizeof(float2), st>>>(b.pd, b.nprob, sino, out, H,
                                                                                         b.tw, b.Lmax);
}
void batch_rhs(const BatchDev& b, float mu, float lambda, const float* ifkt, const float* dx, const float* bx,
               const float* dy, const float* by, float* rhs, cudaStream_t st)
{
    k_batch_rhs<<<(unsigned)b.n_ew, 256, 0, st>>>(b.pd, b.nprob, mu, lambda, ifkt, dx, bx, dy, by, rhs);
}
void batch_resid(const BatchDev& b, float mu, float lambda, const float* rhs, const float* iukt, const float* uk,
                 float* r, float* p, double* part, cudaStream_t st)
{
    k_batch_resid<<<(unsigned)b.n_ew, 256, 0, st>>>(b.pd, b.nprob, mu, lambda, rhs, iukt, uk, r, p, part);
}
void batch_apply(const BatchDev& b, float mu, float lambda, const float* irpt, const float* p, float* Ap,
                 double* part, cudaStream_t st)
{
    k_batch_apply<<<(unsigned)b.n_ew, 256, 0, st>>>(b.pd, b.nprob, mu, lambda, irpt, p, Ap, part);
}
void batch_update(const BatchDev& b, const float* p, const float* Ap, float* uk, float* r, const double* alpha,
                  double* part, cudaStream_t st)
{
    k_batch_update<<<(unsigned)b.n_ew, 256, 0, st>>>(b.pd, b.nprob, p, Ap, uk, r, alpha, part);
}
void batch_pupdate(const BatchDev& b, const float* r, float* p, const double* beta, cudaStream_t st)
{
    k_batch_pupdate<<<(unsigned)b.n_ew, 256, 0, st>>>(b.pd, b.nprob, r, p, beta);
}
void batch_shrink(const BatchDev& b, float lambda, const float* uk, float* dx, float* bx, float* dy, float* by,
                  cudaStream_t st)
{
    k_batch_shrink<<<(unsigned)b.n_ew, 256, 0, st>>>(b.pd, b.nprob, lambda, uk, dx, bx, dy, by);
}
void batch_fk(const BatchDev& b, float* fk, const float* f, const float* ruk, cudaStream_t st)
{
    k_batch_fk<<<4096, 256, 0, st>>>(b.sino_total, fk, f, ruk);
}
void batch_diff(const BatchDev& b, const float* a, const float* c, float* out, cudaStream_t st)
{
    k_batch_diff<<<4096, 256, 0, st>>>(b.sino_total, a, c, out);
}
void batch_sino_axpy(const BatchDev& b, const double* alpha, const float* x, float* y, cudaStream_t st)
{
    k_batch_sino_axpy<<<dim3(64, b.nprob), 256, 0, st>>>(b.pd, alpha, x, y);
}
void batch_finalize(const BatchDev& b, int which, const double* part, double* rsold, double* alpha, double* beta,
                    cudaStream_t st)
{
    k_batch_finalize<<<b.nprob, 256, 0, st>>>(b.pd, b.nprob, b.n_ew, which, part, rsold, alpha, beta);
}

}  // namespace acu

// =============================================================================
// host side: the batch object and its C ABI
// =============================================================================
using namespace acu;

struct acu_batch {
    acu_ctx* ctx = nullptr;   // stream, error slot, own stream for captures
    int nprob = 0;
    std::vector<int> N, T, wpu;
    std::vector<ProbDesc> desc;       // in caller order
    std::vector<int> order;           // execution order (largest work first) -> caller index
    BatchDev dev;
    DevBuf d_pd, d_sc_bp, d_sc_fp, d_xsc_bp, d_xsc_fp, d_cm, d_fh, d_fhx, d_tw, d_counter;
    DevBuf f, fk, ruk, rp, q, uk, dx, dy, bx, by, rhs, r, p, Ap, tmp, part, rsold, alpha, beta, it_img;
    DevBuf io_in, io_out;
    cudaGraphExec_t graph = nullptr, graph_inc = nullptr;
    std::string graph_key;
    bool tuned = false;
    int refresh = 5;   // radon(uk) recomputed every refresh-th outer iteration (ACU_OPT_RADON_REFRESH)
    ~acu_batch()
    {
        if (graph) cudaGraphExecDestroy(graph);
        if (graph_inc) cudaGraphExecDestroy(graph_inc);
        if (ctx) acu_ctx_destroy(ctx);
    }
};

namespace {

int berr(acu_batch* b, int code, const char* msg)
{
    return set_err(b ? b->ctx : nullptr, code, "%s", msg);
}

#define BCK(call) CK(b->ctx, call)

// One Bregman outer iteration of every problem (tv_hpc.F90:205-353), ruk =
// radon(uk) on entry.
// One outer iteration, with the uniform solver's two restructurings: the
// initial residual from one backprojection of fk - radon(uk), and radon(uk)
// carried through the CG updates unless `full` (or refresh == 1).
void batch_outer(acu_batch* b, cudaStream_t st, int ninner, int ncg, float lambda, float mu, bool full)
{
    const bool carry = b->refresh != 1;
    const BatchDev& d = b->dev;
    auto F = [](DevBuf& x) { return x.as<float>(); };
    auto D = [](DevBuf& x) { return x.as<double>(); };
    auto iradon = [&](const float* s, float* img) {
        batch_filter(d, s, F(b->q), st);
        batch_backproject(d, F(b->q), img, 1, st);
    };
    for (int ji = 1; ji <= ninner; ++ji) {
        if (ji > 1 && !carry) batch_radon(d, F(b->uk), F(b->ruk), 0, st);
        batch_diff(d, F(b->fk), F(b->ruk), F(b->rp), st);
        iradon(F(b->rp), F(b->tmp));
        batch_rhs(d, mu, lambda, F(b->tmp), F(b->dx), F(b->bx), F(b->dy), F(b->by), F(b->rhs), st);
        batch_resid(d, mu, lambda, F(b->rhs), nullptr, F(b->uk), F(b->r), F(b->p), D(b->part), st);
        batch_finalize(d, 0, D(b->part), D(b->rsold), D(b->alpha), D(b->beta), st);
        for (int k = 0; k < ncg; ++k) {
            batch_radon(d, F(b->p), F(b->rp), 0, st);
            iradon(F(b->rp), F(b->tmp));
            batch_apply(d, mu, lambda, F(b->tmp), F(b->p), F(b->Ap), D(b->part), st);
            batch_finalize(d, 1, D(b->part), D(b->rsold), D(b->alpha), D(b->beta), st);
            batch_update(d, F(b->p), F(b->Ap), F(b->uk), F(b->r), D(b->alpha), D(b->part), st);
            if (carry) batch_sino_axpy(d, D(b->alpha), F(b->rp), F(b->ruk), st);
            batch_finalize(d, 2, D(b->part), D(b->rsold), D(b->alpha), D(b->beta), st);
            batch_pupdate(d, F(b->r), F(b->p), D(b->beta), st);
        }
        batch_shrink(d, lambda, F(b->uk), F(b->dx), F(b->bx), F(b->dy), F(b->by), st);
    }
    if (full || !carry) batch_radon(d, F(b->uk), F(b->ruk), 0, st);
    batch_fk(d, F(b->fk), F(b->f), F(b->ruk), st);
}

// Picks the projector's warps per block by timing each candidate once on the
// batch (zero image); tune_all does the same for the backprojection's tile
// height.
int autotune(acu_batch* b)
{
    if (b->tuned) return ACU_OK;
    cudaStream_t st = b->ctx->stream;
    cudaEvent_t e0, e1;
    BCK(cudaEventCreate(&e0));
    BCK(cudaEventCreate(&e1));
    float best = 1e30f;
    int bw = 4;
    for (int w : {2, 4, 8, 16}) {
        b->dev.radon_warps = w;
        batch_radon(b->dev, b->uk.as<float>(), b->rp.as<float>(), 0, st);   // warm
        BCK(cudaEventRecord(e0, st));
        batch_radon(b->dev, b->uk.as<float>(), b->rp.as<float>(), 0, st);
        BCK(cudaEventRecord(e1, st));
        BCK(cudaEventSynchronize(e1));
        float ms = 0;
        BCK(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) { best = ms; bw = w; }
    }
    b->dev.radon_warps = bw;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->tuned = true;
    return ACU_OK;
}

// copy between the caller's problem order (packed) and the execution order
int repack(acu_batch* b, const float* src, float* dst, bool sino, bool to_exec, cudaMemcpyKind kind)
{
    std::vector<long long> caller_off(b->nprob + 1, 0);
    for (int i = 0; i < b->nprob; ++i)
        caller_off[i + 1] = caller_off[i] + (sino ? (long long)b->T[i] * b->N[i] : (long long)b->N[i] * b->N[i]);
    for (int i = 0; i < b->nprob; ++i) {
        const ProbDesc& d = b->desc[i];
        const long long exec_off = sino ? d.sino : d.img;
        const long long n = caller_off[i + 1] - caller_off[i];
        const float* s = to_exec ? src + caller_off[i] : src + exec_off;
        float* t = to_exec ? dst + exec_off : dst + caller_off[i];
        BCK(cudaMemcpyAsync(t, s, sizeof(float) * n, kind, b->ctx->stream));
    }
    return ACU_OK;
}

}  // namespace

extern "C" {

int acu_batch_create(acu_batch** out, int nprob, const int* nimage, const int* ntheta, const float* theta_concat,
                     const int* wpu)
{
    if (!out) return set_err(nullptr, ACU_ERR_INVALID, "null output pointer");
    *out = nullptr;
    if (nprob < 1 || !nimage || !ntheta || !theta_concat || !wpu)
        return set_err(nullptr, ACU_ERR_INVALID, "invalid batch description");
    for (int i = 0; i < nprob; ++i)
        if (nimage[i] < 3 || nimage[i] > 46340 || ntheta[i] < 1)
            return set_err(nullptr, ACU_ERR_INVALID, "problem %d: invalid geometry N=%d T=%d", i, nimage[i], ntheta[i]);
    std::unique_ptr<acu_batch> b(new (std::nothrow) acu_batch());
    if (!b) return set_err(nullptr, ACU_ERR_NOMEM, "host allocation failed");
    int rc = acu_ctx_create(&b->ctx, 0, 0, nullptr, 0);
    if (rc != ACU_OK) return rc;
    b->nprob = nprob;
    b->N.assign(nimage, nimage + nprob);
    b->T.assign(ntheta, ntheta + nprob);
    b->wpu.assign(wpu, wpu + nprob);
    // execution order: largest work (T * N^2) first, for the persistent kernels
    b->order.resize(nprob);
    std::iota(b->order.begin(), b->order.end(), 0);
    std::stable_sort(b->order.begin(), b->order.end(), [&](int a, int c) {
        return (double)b->T[a] * b->N[a] * b->N[a] > (double)b->T[c] * b->N[c] * b->N[c];
    });
    std::vector<long long> th_off(nprob + 1, 0);
    for (int i = 0; i < nprob; ++i) th_off[i + 1] = th_off[i] + b->T[i];
    int Lmax = 16;
    std::vector<HostTables<float>> tabs(nprob);
    for (int i = 0; i < nprob; ++i) {
        make_tables<float>(b->N[i], b->T[i], theta_concat + th_off[i], b->wpu[i], tabs[i]);
        Lmax = std::max(Lmax, tabs[i].fft_L);
    }
    if (2 * (size_t)Lmax * sizeof(float2) > 227 * 1024)
        return berr(b.get(), ACU_ERR_UNSUPPORTED, "a problem needs an FFT longer than 8192 (grid side > 4097)");
    b->desc.resize(nprob);
    std::vector<float> sc_bp, sc_fp, xsc_bp, xsc_fp, cm, fh, fhx;
    long long img = 0, sino = 0, ir = 0, ib = 0, iff = 0, ie = 0, itr = 0;
    std::vector<ProbDesc> exec_desc;
    for (int k = 0; k < nprob; ++k) {
        const int i = b->order[k];
        const HostTables<float>& h = tabs[i];
        ProbDesc d{};
        d.N = b->N[i];
        d.T = b->T[i];
        d.L = h.fft_L;
        d.lg = h.fft_log2L;
        d.mid = h.mid;
        d.nbx = (d.N + 31) / 32;
        d.img = img;
        d.sino = sino;
        d.sc = (long long)sc_bp.size();
        d.cm = (long long)cm.size();
        d.fh = (long long)fh.size();
        d.it_radon = ir;
        d.it_bp = ib;
        d.it_fft = iff;
        d.it_ew = ie;
        sc_bp.insert(sc_bp.end(), h.sc_bp.begin(), h.sc_bp.end());
        sc_fp.insert(sc_fp.end(), h.sc_fp.begin(), h.sc_fp.end());
        xsc_bp.insert(xsc_bp.end(), h.xsc_bp.begin(), h.xsc_bp.end());   // 4 per angle: index sc / 2
        xsc_fp.insert(xsc_fp.end(), h.xsc_fp.begin(), h.xsc_fp.end());
        cm.insert(cm.end(), h.cmask.begin(), h.cmask.end());
        fh.insert(fh.end(), h.fft_h.begin(), h.fft_h.end());
        fhx.insert(fhx.end(), h.fft_h_x.begin(), h.fft_h_x.end());
        img += (long long)d.N * d.N;
        sino += (long long)d.T * d.N;
        ir += (long long)d.T * d.nbx;
        ib += (long long)((d.N + 31) / 32) * ((d.N + 3) / 4);   // rows of the smallest tile height
        iff += (d.T + 1) / 2;
        ie += ((long long)d.N * d.N + EWB - 1) / EWB;
        d.it_tr = itr;
        itr += (long long)((d.N + 31) / 32) * ((d.N + 31) / 32);
        b->desc[i] = d;
        exec_desc.push_back(d);
    }
    if (ir > 0x7fffffff || ib > 0x7fffffff) return berr(b.get(), ACU_ERR_UNSUPPORTED, "batch too large for the work lists");
    // twiddles of the largest transform
    std::vector<float2> tw(Lmax);
    for (int k = 0; k < Lmax; ++k) {
        const double a = -2.0 * 3.14159265358979323846 * (double)k / (double)Lmax;
        tw[k] = make_float2((float)std::cos(a), (float)std::sin(a));
    }
    acu_ctx* c = b->ctx;
    auto up = [&](DevBuf& buf, const void* src, size_t bytes) -> int {
        CK(c, buf.ensure(bytes));
        CK(c, cudaMemcpy(buf.p, src, bytes, cudaMemcpyHostToDevice));
        return ACU_OK;
    };
    CKRET(up(b->d_pd, exec_desc.data(), sizeof(ProbDesc) * nprob));
    CKRET(up(b->d_sc_bp, sc_bp.data(), sizeof(float) * sc_bp.size()));
    CKRET(up(b->d_sc_fp, sc_fp.data(), sizeof(float) * sc_fp.size()));
    CKRET(up(b->d_xsc_bp, xsc_bp.data(), sizeof(float) * xsc_bp.size()));
    CKRET(up(b->d_xsc_fp, xsc_fp.data(), sizeof(float) * xsc_fp.size()));
    CKRET(up(b->d_cm, cm.data(), sizeof(float) * cm.size()));
    CKRET(up(b->d_fh, fh.data(), sizeof(float) * fh.size()));
    CKRET(up(b->d_fhx, fhx.data(), sizeof(float) * fhx.size()));
    CKRET(up(b->d_tw, tw.data(), sizeof(float2) * tw.size()));
    CK(c, b->d_counter.ensure(sizeof(int) * 8));
    BatchDev& d = b->dev;
    d.nprob = nprob;
    d.pd = b->d_pd.as<ProbDesc>();
    d.sc_bp = b->d_sc_bp.as<float>();
    d.sc_fp = b->d_sc_fp.as<float>();
    d.xsc_bp = b->d_xsc_bp.as<float4>();
    d.xsc_fp = b->d_xsc_fp.as<float4>();
    d.cmask = b->d_cm.as<float>();
    d.fft_h = b->d_fh.as<float>();
    d.fft_h_x = b->d_fhx.as<float>();
    d.tw = b->d_tw.as<float2>();
    d.Lmax = Lmax;
    d.n_radon = ir;
    d.n_bp = ib;
    d.n_fft = iff;
    d.n_ew = ie;
    d.n_tr = itr;
    d.img_total = img;
    d.sino_total = sino;
    d.counter = b->d_counter.as<int>();
    // the work list of the backprojection depends on the tile height chosen by
    // the autotuner: items of every problem are recomputed for it at launch
    *out = b.release();
    return ACU_OK;
}

int acu_batch_destroy(acu_batch* b)
{
    if (!b) return ACU_OK;
    cudaStreamSynchronize(b->ctx ? b->ctx->stream : nullptr);
    delete b;
    return ACU_OK;
}

int acu_batch_set_stream(acu_batch* b, void* stream)
{
    if (!b) return set_err(nullptr, ACU_ERR_INVALID, "null batch");
    return acu_set_stream(b->ctx, stream);
}

const char* acu_batch_last_error(const acu_batch* b) { return acu_last_error(b ? b->ctx : nullptr); }

}  // extern "C"

namespace {

// backprojection items per problem for the chosen tile height
int set_bp_rows(acu_batch* b, int rows)
{
    b->dev.bp_rows = rows;
    std::vector<ProbDesc> ex(b->nprob);
    long long ib = 0;
    for (int k = 0; k < b->nprob; ++k) {
        ProbDesc d = b->desc[b->order[k]];
        d.it_bp = ib;
        ib += (long long)((d.N + 31) / 32) * ((d.N + rows - 1) / rows);
        ex[k] = d;
        b->desc[b->order[k]].it_bp = d.it_bp;
    }
    b->dev.n_bp = ib;
    CK(b->ctx, cudaMemcpy(b->d_pd.p, ex.data(), sizeof(ProbDesc) * b->nprob, cudaMemcpyHostToDevice));
    return ACU_OK;
}

int ensure_state(acu_batch* b)
{
    acu_ctx* c = b->ctx;
    const size_t ni = sizeof(float) * (size_t)b->dev.img_total, ns = sizeof(float) * (size_t)b->dev.sino_total;
    for (DevBuf* x : {&b->f, &b->fk, &b->ruk, &b->rp, &b->q}) CK(c, x->ensure(ns));
    for (DevBuf* x : {&b->uk, &b->dx, &b->dy, &b->bx, &b->by, &b->rhs, &b->r, &b->p, &b->Ap, &b->tmp, &b->it_img})
        CK(c, x->ensure(ni));
    b->dev.IT = b->it_img.as<float>();
    CK(c, b->part.ensure(sizeof(double) * (size_t)b->dev.n_ew));
    for (DevBuf* x : {&b->rsold, &b->alpha, &b->beta}) CK(c, x->ensure(sizeof(double) * b->nprob));
    return ACU_OK;
}

int tune_all(acu_batch* b)
{
    if (b->tuned) return ACU_OK;
    CKRET(ensure_state(b));
    CK(b->ctx, cudaMemsetAsync(b->uk.p, 0, sizeof(float) * b->dev.img_total, b->ctx->stream));
    CK(b->ctx, cudaMemsetAsync(b->q.p, 0, sizeof(float) * b->dev.sino_total, b->ctx->stream));
    // the backprojection work list must match the tile height while timing
    cudaStream_t st = b->ctx->stream;
    cudaEvent_t e0, e1;
    CK(b->ctx, cudaEventCreate(&e0));
    CK(b->ctx, cudaEventCreate(&e1));
    float best = 1e30f;
    int br = 8;
    for (int rr : {4, 8, 16}) {
        CKRET(set_bp_rows(b, rr));
        batch_backproject(b->dev, b->q.as<float>(), b->tmp.as<float>(), 1, st);
        CK(b->ctx, cudaEventRecord(e0, st));
        batch_backproject(b->dev, b->q.as<float>(), b->tmp.as<float>(), 1, st);
        CK(b->ctx, cudaEventRecord(e1, st));
        CK(b->ctx, cudaEventSynchronize(e1));
        float ms = 0;
        CK(b->ctx, cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) { best = ms; br = rr; }
    }
    CKRET(set_bp_rows(b, br));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->tuned = false;
    CKRET(autotune(b));   // projector warps per block (marks the batch tuned)
    CKRET(set_bp_rows(b, br));
    return ACU_OK;
}

int batch_solve(acu_batch* b, const float* d_f_exec, int ninner, int nouter, int ncg, float lambda, float mu,
                float* d_tv_exec, float* d_fbp_exec)
{
    acu_ctx* c = b->ctx;
    CKRET(tune_all(b));
    cudaStream_t st = c->stream;
    const BatchDev& d = b->dev;
    auto F = [](DevBuf& x) { return x.as<float>(); };
    CK(c, cudaMemcpyAsync(b->f.p, d_f_exec, sizeof(float) * d.sino_total, cudaMemcpyDeviceToDevice, st));
    batch_filter(d, F(b->f), F(b->q), st);
    batch_backproject(d, F(b->q), F(b->uk), 1, st);
    if (d_fbp_exec) CK(c, cudaMemcpyAsync(d_fbp_exec, b->uk.p, sizeof(float) * d.img_total, cudaMemcpyDeviceToDevice, st));
    for (DevBuf* x : {&b->dx, &b->dy, &b->bx, &b->by}) CK(c, cudaMemsetAsync(x->p, 0, sizeof(float) * d.img_total, st));
    CK(c, cudaMemcpyAsync(b->fk.p, b->f.p, sizeof(float) * d.sino_total, cudaMemcpyDeviceToDevice, st));
    batch_radon(d, F(b->uk), F(b->ruk), 0, st);
    CKLAUNCH(c);
    if (nouter > 0) {
        char key[160];
        snprintf(key, sizeof key, "%d/%d/%.9g/%.9g/%d/%d/%d/%d", ninner, ncg, (double)lambda, (double)mu,
                 d.radon_warps, d.bp_rows, d.exact, b->refresh);
        if (!b->graph || b->graph_key != key) {
            for (cudaGraphExec_t* gx : {&b->graph, &b->graph_inc})
                if (*gx) {
                    cudaGraphExecDestroy(*gx);
                    *gx = nullptr;
                }
            // graph: radon(uk) recomputed at the end; graph_inc: carried
            for (int which = 0; which < (b->refresh == 1 ? 1 : 2); ++which) {
                cudaGraph_t g;
                CK(c, cudaStreamBeginCapture(c->own_stream, cudaStreamCaptureModeThreadLocal));
                batch_outer(b, c->own_stream, ninner, ncg, lambda, mu, which == 0);
                cudaError_t e = cudaStreamEndCapture(c->own_stream, &g);
                if (e != cudaSuccess)
                    return set_err(c, ACU_ERR_CUDA, "batch graph capture failed: %s", cudaGetErrorString(e));
                cudaGraphExec_t* gx = which == 0 ? &b->graph : &b->graph_inc;
                e = cudaGraphInstantiate(gx, g, 0);
                cudaGraphDestroy(g);
                if (e != cudaSuccess) {
                    *gx = nullptr;
                    return set_err(c, ACU_ERR_CUDA, "batch graph instantiate failed: %s", cudaGetErrorString(e));
                }
            }
            b->graph_key = key;
        }
        for (int k = 1; k <= nouter; ++k) {
            const bool full = b->refresh == 1 || (b->refresh > 1 && k % b->refresh == 0);
            CK(c, cudaGraphLaunch(full ? b->graph : b->graph_inc, st));
        }
    }
    CK(c, cudaMemcpyAsync(d_tv_exec, b->uk.p, sizeof(float) * d.img_total, cudaMemcpyDeviceToDevice, st));
    return ACU_OK;
}

}  // namespace

extern "C" {

// f: concatenated sinograms in the caller's problem order (problem i: T_i*N_i),
// tv / fbp: concatenated images (N_i*N_i).  Host pointers.
int acu_batch_tvopt(acu_batch* b, const float* f, int ninner, int nouter, int ncg, float lambda, float mu, float* tv,
                    float* fbp)
{
    if (!b) return set_err(nullptr, ACU_ERR_INVALID, "null batch");
    if (!f || !tv) return berr(b, ACU_ERR_INVALID, "null array");
    if (ninner < 0 || nouter < 0 || ncg < 0) return berr(b, ACU_ERR_INVALID, "iteration counts must be >= 0");
    if (lambda == 0.0f) return berr(b, ACU_ERR_INVALID, "lambda must be non-zero (shrink threshold 1/lambda)");
    acu_ctx* c = b->ctx;
    const size_t ns = (size_t)b->dev.sino_total, ni = (size_t)b->dev.img_total;
    CK(c, b->io_in.ensure(sizeof(float) * ns));
    CK(c, b->io_out.ensure(sizeof(float) * ni * 2));
    CKRET(repack(b, f, b->io_in.as<float>(), true, true, cudaMemcpyHostToDevice));
    float* d_tv = b->io_out.as<float>();
    float* d_fbp = d_tv + ni;
    CKRET(batch_solve(b, b->io_in.as<float>(), ninner, nouter, ncg, lambda, mu, d_tv, d_fbp));
    CKRET(repack(b, d_tv, tv, false, false, cudaMemcpyDeviceToHost));
    if (fbp) CKRET(repack(b, d_fbp, fbp, false, false, cudaMemcpyDeviceToHost));
    CK(c, cudaStreamSynchronize(c->stream));
    return ACU_OK;
}

// Single operators of the batch on host buffers (for checks): op 0 radon
// (images -> sinograms), 1 iradon (sinograms -> images).
int acu_batch_op(acu_batch* b, int op, const float* in, float* out)
{
    if (!b) return set_err(nullptr, ACU_ERR_INVALID, "null batch");
    if (!in || !out || (op != 0 && op != 1)) return berr(b, ACU_ERR_INVALID, "invalid operator call");
    acu_ctx* c = b->ctx;
    CKRET(tune_all(b));
    const size_t ns = (size_t)b->dev.sino_total, ni = (size_t)b->dev.img_total;
    CK(c, b->io_in.ensure(sizeof(float) * std::max(ns, ni)));
    CK(c, b->io_out.ensure(sizeof(float) * std::max(ns, ni) * 2));
    float* din = b->io_in.as<float>();
    float* dout = b->io_out.as<float>();
    CKRET(repack(b, in, din, op == 1, true, cudaMemcpyHostToDevice));
    if (op == 0) {
        batch_radon(b->dev, din, dout, 0, c->stream);
    } else {
        batch_filter(b->dev, din, b->q.as<float>(), c->stream);
        batch_backproject(b->dev, b->q.as<float>(), dout, 1, c->stream);
    }
    CKLAUNCH(c);
    CKRET(repack(b, dout, out, op == 0, false, cudaMemcpyDeviceToHost));
    CK(c, cudaStreamSynchronize(c->stream));
    return ACU_OK;
}

int acu_batch_tuning(const acu_batch* b, int* radon_warps, int* bp_rows)
{
    if (!b || !radon_warps || !bp_rows) return set_err(nullptr, ACU_ERR_INVALID, "null argument");
    *radon_warps = b->dev.radon_warps;
    *bp_rows = b->dev.bp_rows;
    return ACU_OK;
}

int acu_batch_set_option(acu_batch* b, int option, int value)
{
    if (!b) return set_err(nullptr, ACU_ERR_INVALID, "null batch");
    if (option == ACU_OPT_RADON_REFRESH) {
        if (value < 0) return berr(b, ACU_ERR_INVALID, "ACU_OPT_RADON_REFRESH must be >= 0");
        b->refresh = value;
        return ACU_OK;
    }
    if (option != ACU_OPT_POSITIONS)
        return berr(b, ACU_ERR_INVALID, "acu_batch_set_option: only ACU_OPT_POSITIONS and ACU_OPT_RADON_REFRESH");
    if (value != 0 && value != 1) return berr(b, ACU_ERR_INVALID, "ACU_OPT_POSITIONS must be 0 or 1");
    b->dev.exact = value;
    return ACU_OK;
}

}  // extern "C"
