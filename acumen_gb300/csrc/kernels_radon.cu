// Radon-transform kernels: pixel-driven backprojection (iradon's second half),
// the bilinear ray-sum projector (radon), its exact transpose, and the direct
// ramp-filter convolution (iradon's first half).
//
// Arrays are in lane layout (common.cuh): V slices of one group interleaved,
// so each thread carries V slices through one geometry evaluation.
#include "common.cuh"
#include "kernels.h"

#include <cstring>

namespace acu {

// ---------------------------------------------------------------------------
// Backprojection: tomography/tv_hpc.F90:107-123.
//   img(jx,jy) = cmask(jx,jy) * sum_theta [ q(y1)*(y2-yr) + q(y2)*(yr-y1) ]
//   yr = sin(c)*(jx-m) + cos(c)*(jy-m) + m,  c = pi*(90-theta)/180,
//   taps used only when y1 = floor(yr) > 1 and y2 = y1+1 < N+1.
// One thread per pixel and slice group; angles summed in the reference's
// order.  Pixels whose mask is zero are written as 0 without the angle loop.
// ---------------------------------------------------------------------------
template <typename Real, int V, int GPT>
__global__ void __launch_bounds__(256) k_backproject(const Real* __restrict__ q,
                                                     const Real* __restrict__ cmask,
                                                     const Real* __restrict__ sc, Real* __restrict__ img,
                                                     int N, int T, Real mid)
{
    const int jx = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int jy = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int g0 = blockIdx.z * GPT;
    if (jx > N || jy > N) return;
    const size_t pix = (size_t)(jy - 1) * N + (jx - 1);
    const Real cm = cmask[pix];
    Lanes<Real, V> acc[GPT];
#pragma unroll
    for (int k = 0; k < GPT; ++k)
#pragma unroll
        for (int v = 0; v < V; ++v) acc[k].v[v] = Real(0);
    if (cm != Real(0)) {
        const Real dx = (Real)jx - mid, dy = (Real)jy - mid;
        const Real* qg = q + (size_t)g0 * T * N * V;
        for (int t = 0; t < T; ++t) {
            const Lanes<Real, 2> scp = ld_lanes<Real, 2>(sc + 2 * t);
            const Real s = scp.v[0], c = scp.v[1];
            const Real yr = add_rn(add_rn(mul_rn(s, dx), mul_rn(c, dy)), mid);
            const Real y1f = rfloor(yr);
            const int y1 = (int)y1f;
            if (y1 > 1 && y1 < N) {
                const Real wl = add_rn(y1f, Real(1)) - yr;
                const Real wh = yr - y1f;
#pragma unroll
                for (int k = 0; k < GPT; ++k) {
                    const Real* row = qg + ((size_t)(k * T + t) * N + (y1 - 1)) * V;
                    const Lanes<Real, V> a = ld_lanes<Real, V>(row);
                    const Lanes<Real, V> b = ld_lanes<Real, V>(row + V);
#pragma unroll
                    for (int v = 0; v < V; ++v) acc[k].v[v] = fma(b.v[v], wh, fma(a.v[v], wl, acc[k].v[v]));
                }
            }
        }
    }
#pragma unroll
    for (int k = 0; k < GPT; ++k) {
#pragma unroll
        for (int v = 0; v < V; ++v) acc[k].v[v] = cm * acc[k].v[v];
        st_lanes<Real, V>(img + ((size_t)(g0 + k) * N * N + pix) * V, acc[k]);
    }
}

// acc += a wl + b wh slice by slice, as two fused multiply-adds in that order;
// four slices as paired FMAs (fma.rn.f32x2, each half rounded as fmaf), which
// halves the instructions of the backprojection's inner loop.
template <int V>
__device__ __forceinline__ void lerp_acc(Lanes<float, V>& acc, const Lanes<float, V>& a, const Lanes<float, V>& b,
                                         float wl, float wh)
{
    if constexpr (V == 4) {
        const float2 WL = make_float2(wl, wl), WH = make_float2(wh, wh);
        float2 lo = make_float2(acc.v[0], acc.v[1]), hi = make_float2(acc.v[2], acc.v[3]);
        lo = fma2(make_float2(a.v[0], a.v[1]), WL, lo);
        hi = fma2(make_float2(a.v[2], a.v[3]), WL, hi);
        lo = fma2(make_float2(b.v[0], b.v[1]), WH, lo);
        hi = fma2(make_float2(b.v[2], b.v[3]), WH, hi);
        acc.v[0] = lo.x;
        acc.v[1] = lo.y;
        acc.v[2] = hi.x;
        acc.v[3] = hi.y;
    } else {
#pragma unroll
        for (int v = 0; v < V; ++v) acc.v[v] = fmaf(b.v[v], wh, fmaf(a.v[v], wl, acc.v[v]));
    }
}

// k_backproject in single precision with the per-angle (sin, cos) read from
// the launch parameters (constant-cache broadcast; T <= BP_TMAX).
template <int V, int GPT>
__global__ void __launch_bounds__(256) k_backproject_ct(const float* __restrict__ q,
                                                        const float* __restrict__ cmask,
                                                        const __grid_constant__ BpTable tab,
                                                        float* __restrict__ img, int N, int T, float mid)
{
    const int jx = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int jy = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int g0 = blockIdx.z * GPT;
    if (jx > N || jy > N) return;
    const size_t pix = (size_t)(jy - 1) * N + (jx - 1);
    const float cm = cmask[pix];
    Lanes<float, V> acc[GPT];
#pragma unroll
    for (int k = 0; k < GPT; ++k)
#pragma unroll
        for (int v = 0; v < V; ++v) acc[k].v[v] = 0.f;
    if (cm != 0.f) {
        const float dx = (float)jx - mid, dy = (float)jy - mid;
        const float* qg = q + (size_t)g0 * T * N * V;
        for (int t = 0; t < T; ++t) {
            const float4 scp = tab.v[t];
            const float s = scp.x, c = scp.y;
            const float yr = add_rn(add_rn(mul_rn(s, dx), mul_rn(c, dy)), mid);
            const float y1f = rfloor(yr);
            const int y1 = (int)y1f;
            if (y1 > 1 && y1 < N) {
                const float wl = add_rn(y1f, 1.f) - yr;
                const float wh = yr - y1f;
#pragma unroll
                for (int k = 0; k < GPT; ++k) {
                    const float* row = qg + ((size_t)(k * T + t) * N + (y1 - 1)) * V;
                    const Lanes<float, V> a = ld_lanes<float, V>(row);
                    const Lanes<float, V> b = ld_lanes<float, V>(row + V);
                    lerp_acc<V>(acc[k], a, b, wl, wh);
                }
            }
        }
    }
#pragma unroll
    for (int k = 0; k < GPT; ++k) {
#pragma unroll
        for (int v = 0; v < V; ++v) acc[k].v[v] = cm * acc[k].v[v];
        st_lanes<float, V>(img + ((size_t)(g0 + k) * N * N + pix) * V, acc[k]);
    }
}

// The same backprojection with exact sample positions (option 8): the
// coordinate yr = s*dx + c*dy + mid is evaluated from the split FP64 angle
// tables, so its cell and fraction agree with double precision to ~1e-7 px
// instead of the ~1e-4 px of the reference's single-precision rounding at
// grid sides of a few thousand.  Sums, weights and order are as above.
// Per-angle table reads of the exact backprojection: from global memory, or
// from a kernel parameter (constant bank: a warp-uniform read is a constant-
// cache broadcast and takes no L1 data-pipe wavefronts).
struct TabGlobal {
    const float4* p;
    __device__ __forceinline__ float4 operator()(int t) const { return __ldg(p + t); }
};
struct TabParam {
    const BpTable* p;
    __device__ __forceinline__ float4 operator()(int t) const { return p->v[t]; }
};

template <int V, int GPT, typename Tab>
__device__ __forceinline__ void bp_exact_body(const float* __restrict__ q, const float* __restrict__ cmask, Tab tab,
                                              float* __restrict__ img, int N, int T, float mid)
{
    const int jx = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int jy = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int g0 = blockIdx.z * GPT;
    if (jx > N || jy > N) return;
    const size_t pix = (size_t)(jy - 1) * N + (jx - 1);
    const float cm = cmask[pix];
    Lanes<float, V> acc[GPT];
#pragma unroll
    for (int k = 0; k < GPT; ++k)
#pragma unroll
        for (int v = 0; v < V; ++v) acc[k].v[v] = 0.f;
    if (cm != 0.f) {
        const float dx = (float)jx - mid, dy = (float)jy - mid;
        const float* qg = q + (size_t)g0 * T * N * V;
        for (int t = 0; t < T; ++t) {
            const float4 x = tab(t);
            float cell, wh;
            exact_coord(x.x, x.y, x.z, x.w, dx, dy, mid, cell, wh);
            const int y1 = (int)cell;
            if (y1 > 1 && y1 < N) {
                const float wl = 1.f - wh;
#pragma unroll
                for (int k = 0; k < GPT; ++k) {
                    const float* row = qg + ((size_t)(k * T + t) * N + (y1 - 1)) * V;
                    const Lanes<float, V> a = ld_lanes<float, V>(row);
                    const Lanes<float, V> b = ld_lanes<float, V>(row + V);
                    lerp_acc<V>(acc[k], a, b, wl, wh);
                }
            }
        }
    }
#pragma unroll
    for (int k = 0; k < GPT; ++k) {
#pragma unroll
        for (int v = 0; v < V; ++v) acc[k].v[v] = cm * acc[k].v[v];
        st_lanes<float, V>(img + ((size_t)(g0 + k) * N * N + pix) * V, acc[k]);
    }
}

template <int V, int GPT>
__global__ void __launch_bounds__(256) k_backproject_exact(const float* __restrict__ q,
                                                           const float* __restrict__ cmask,
                                                           const float4* __restrict__ xsc,
                                                           float* __restrict__ img, int N, int T, float mid)
{
    bp_exact_body<V, GPT>(q, cmask, TabGlobal{xsc}, img, N, T, mid);
}

template <int V, int GPT>
__global__ void __launch_bounds__(256) k_backproject_exact_ct(const float* __restrict__ q,
                                                              const float* __restrict__ cmask,
                                                              const __grid_constant__ BpTable tab,
                                                              float* __restrict__ img, int N, int T, float mid)
{
    bp_exact_body<V, GPT>(q, cmask, TabParam{&tab}, img, N, T, mid);
}

// ---- backprojection with the sinogram bins staged in shared memory by the
// bulk-copy (TMA) engine.  A block is a tile of 32 x 8 pixels (one pixel and
// one 4-slice group per thread, exact positions, angle table in the launch
// parameters).  For every angle, the bins the tile's pixels interpolate lie
// between the cells of its four corners (the position is affine in the
// pixel): that range plus one bin each side, at most 32|s| + 8|c| + 4 <= 37
// bins of 16 bytes, is one contiguous piece of the filtered sinogram row.
// The lanes of warp 0 copy the pieces of BPT_A angles per stage (one angle
// each) with cp.async.bulk into one of two shared buffers, completing an
// mbarrier with the byte count; all threads wait on it (bounded), interpolate
// from shared memory and synchronise, and the next stage's copies overlap the
// current stage's arithmetic.  Positions, taps, weights and summation order are those
// of k_backproject_exact_ct: identical images.  A wait that gives up writes NaN
// into the block's pixels (the results can never pass for valid), after
// waiting, again bounded, for the block's copies in flight.
constexpr int BPT_A = 24;      // angles per stage
constexpr int BPT_BINS = 40;   // staged bins per angle (>= 37)

__device__ __forceinline__ unsigned smem_u32(const void* p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(bar), "r"(parity)
                 : "memory");
    return ok != 0;
}
// bounded wait: false if the phase did not complete within `limit` polls
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity, int limit)
{
    for (int i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

struct BptStage {
    float4 bins[BPT_A][BPT_BINS];
    int lo[BPT_A];    // 1-based first staged bin of each angle
    int cnt[BPT_A];   // staged bins of each angle
};

__global__ void __launch_bounds__(256) k_backproject_tma(const float* __restrict__ q, const float* __restrict__ cmask,
                                                         const __grid_constant__ BpTable tab,
                                                         float* __restrict__ img, int N, int T, float mid)
{
    constexpr int V = 4;
    __shared__ __align__(128) BptStage st[2];
    __shared__ __align__(8) unsigned long long bar[2];
    const int tid = threadIdx.y * 32 + threadIdx.x;
    const int jx = blockIdx.x * 32 + threadIdx.x + 1;
    const int jy = blockIdx.y * 8 + threadIdx.y + 1;
    const int g = blockIdx.z;
    // tile corners (clipped to the grid)
    const float cx0 = (float)(blockIdx.x * 32 + 1) - mid, cx1 = (float)min(blockIdx.x * 32 + 32, N) - mid;
    const float cy0 = (float)(blockIdx.y * 8 + 1) - mid, cy1 = (float)min(blockIdx.y * 8 + 8, N) - mid;
    const float* qg = q + (size_t)g * T * N * V;
    const int nstage = (T + BPT_A - 1) / BPT_A;
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar[0])) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar[1])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // warp 0: copies of stage s into buffer s & 1, lane a for angle a
    auto issue = [&](int s) {
        BptStage& b = st[s & 1];
        const int lane = threadIdx.x;
        const int t0 = s * BPT_A, na = min(BPT_A, T - t0);
        int lo = 1, cnt = 0;
        if (lane < na) {
            const float4 x = tab.v[t0 + lane];
            float c, f, cmin = 1e30f, cmax = -1e30f;
            exact_coord(x.x, x.y, x.z, x.w, cx0, cy0, mid, c, f); cmin = fminf(cmin, c); cmax = fmaxf(cmax, c);
            exact_coord(x.x, x.y, x.z, x.w, cx1, cy0, mid, c, f); cmin = fminf(cmin, c); cmax = fmaxf(cmax, c);
            exact_coord(x.x, x.y, x.z, x.w, cx0, cy1, mid, c, f); cmin = fminf(cmin, c); cmax = fmaxf(cmax, c);
            exact_coord(x.x, x.y, x.z, x.w, cx1, cy1, mid, c, f); cmin = fminf(cmin, c); cmax = fmaxf(cmax, c);
            lo = max(1, (int)cmin - 1);
            const int hi = min(N, (int)cmax + 2);
            cnt = max(0, min(hi - lo + 1, BPT_BINS));
            b.lo[lane] = lo;
            b.cnt[lane] = cnt;
        }
        const unsigned bytes = __reduce_add_sync(0xffffffffu, (unsigned)cnt * 16u);
        const unsigned bb = smem_u32(&bar[s & 1]);
        if (lane == 0)
            asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(bb),
                         "r"(bytes)
                         : "memory");
        __syncwarp();
        if (cnt > 0) {
            const float* src = qg + ((size_t)(t0 + lane) * N + (lo - 1)) * V;
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    smem_u32(&b.bins[lane][0])),
                "l"(src), "r"((unsigned)cnt * 16u), "r"(bb)
                : "memory");
        }
    };
    if (threadIdx.y == 0) issue(0);
    const bool inside = jx <= N && jy <= N;
    const size_t pix = inside ? (size_t)(jy - 1) * N + (jx - 1) : 0;
    const float cm = inside ? cmask[pix] : 0.f;
    const float dx = (float)jx - mid, dy = (float)jy - mid;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    bool ok = true;
    int s = 0;
    for (; s < nstage; ++s) {
        if (threadIdx.y == 0 && s + 1 < nstage) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(s + 1);
        }
        // every thread polls; the block leaves together if any gave up
        const bool arrived = mbar_wait(smem_u32(&bar[s & 1]), (unsigned)((s >> 1) & 1), 1 << 22);
        if (!__syncthreads_and(arrived)) {
            ok = false;
            break;
        }
        const BptStage& b = st[s & 1];
        const int t0 = s * BPT_A, na = min(BPT_A, T - t0);
        if (cm != 0.f) {
            for (int a = 0; a < na; ++a) {
                const float4 x = tab.v[t0 + a];
                float cell, wh;
                exact_coord(x.x, x.y, x.z, x.w, dx, dy, mid, cell, wh);
                const int y1 = (int)cell;
                if (y1 > 1 && y1 < N) {
                    const float wl = 1.f - wh;
                    const int k = y1 - b.lo[a];
                    float4 A, B;
                    if (k >= 0 && k + 1 < b.cnt[a]) {
                        A = b.bins[a][k];
                        B = b.bins[a][k + 1];
                    } else {   // outside the staged range (never expected): read the sinogram itself
                        const float* row = qg + ((size_t)(t0 + a) * N + (y1 - 1)) * V;
                        A = __ldg(reinterpret_cast<const float4*>(row));
                        B = __ldg(reinterpret_cast<const float4*>(row) + 1);
                    }
                    acc.x = fmaf(B.x, wh, fmaf(A.x, wl, acc.x));
                    acc.y = fmaf(B.y, wh, fmaf(A.y, wl, acc.y));
                    acc.z = fmaf(B.z, wh, fmaf(A.z, wl, acc.z));
                    acc.w = fmaf(B.w, wh, fmaf(A.w, wl, acc.w));
                }
            }
        }
        __syncthreads();
    }
    if (!ok) {
        // a wait gave up: let the copies already issued land before the block
        // exits (bounded), then mark the block's pixels
        for (int r = s; r < min(s + 2, nstage); ++r) mbar_wait(smem_u32(&bar[r & 1]), (unsigned)((r >> 1) & 1), 1 << 20);
        acc = make_float4(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000), __int_as_float(0x7fc00000),
                          __int_as_float(0x7fc00000));
    }
    if (inside)
        *reinterpret_cast<float4*>(img + ((size_t)g * N * N + pix) * V) =
            ok ? make_float4(cm * acc.x, cm * acc.y, cm * acc.z, cm * acc.w) : acc;
}

// Slice groups per thread: the angle's table entry and the sample position
// are read and formed once for GPT groups (a warp-uniform table load still
// costs the data pipe 32 x its width); each group's sum is unchanged.
template <typename Real, int V, int GPT>
static void backproject_go(const DevGeom<Real>& g, int G, const Real* q, Real* img, cudaStream_t st)
{
    dim3 blk(32, 8), grd((g.N + 31) / 32, (g.N + 7) / 8, G / GPT);
    if constexpr (sizeof(Real) == 4 && V == 4 && GPT == 1) {
        if (g.exact && g.bp_tma && g.bp_param && g.h_xsc_bp && g.T <= BP_TMAX) {
            static thread_local BpTable tab;   // copied into the launch's parameters
            std::memcpy(tab.v, g.h_xsc_bp, sizeof(float4) * g.T);
            k_backproject_tma<<<grd, blk, 0, st>>>(q, g.cmask, tab, img, g.N, g.T, g.mid);
            return;
        }
    }
    if constexpr (sizeof(Real) == 4) {
        if (g.exact) {
            if (g.bp_param && g.h_xsc_bp && g.T <= BP_TMAX) {
                static thread_local BpTable tab;   // copied into the launch's parameters
                std::memcpy(tab.v, g.h_xsc_bp, sizeof(float4) * g.T);
                k_backproject_exact_ct<V, GPT><<<grd, blk, 0, st>>>(q, g.cmask, tab, img, g.N, g.T, g.mid);
            } else {
                k_backproject_exact<V, GPT><<<grd, blk, 0, st>>>(q, g.cmask, g.xsc_bp, img, g.N, g.T, g.mid);
            }
            return;
        }
    }
    if constexpr (sizeof(Real) == 4) {
        if (g.bp_param && g.h_sc_bp && g.T <= BP_TMAX) {
            static thread_local BpTable tab;   // copied into the launch's parameters
            std::memcpy(tab.v, g.h_sc_bp, sizeof(float4) * g.T);
            k_backproject_ct<V, GPT><<<grd, blk, 0, st>>>(q, g.cmask, tab, img, g.N, g.T, g.mid);
            return;
        }
    }
    k_backproject<Real, V, GPT><<<grd, blk, 0, st>>>(q, g.cmask, g.sc_bp, img, g.N, g.T, g.mid);
}

template <typename Real, int V>
void launch_backproject(const DevGeom<Real>& g, int G, const Real* q, Real* img, cudaStream_t st)
{
    if constexpr (V == 4) {
        // auto: one group when the angle table goes in the launch parameters
        // (241 vs 255 ms exact, 236 vs 247 ms reference), else two, which
        // share the table's data-pipe cost (287 vs 334 ms); four need 64
        // registers and are slower in both cases
        const bool param = sizeof(Real) == 4 && g.bp_param && g.T <= BP_TMAX &&
                           (g.exact ? g.h_xsc_bp != nullptr : g.h_sc_bp != nullptr);
        const int want = g.bp_groups > 0 ? g.bp_groups : (param ? 1 : 2);
        if (want >= 4 && G % 4 == 0) return backproject_go<Real, V, 4>(g, G, q, img, st);
        if (want >= 2 && G % 2 == 0) return backproject_go<Real, V, 2>(g, G, q, img, st);
    }
    backproject_go<Real, V, 1>(g, G, q, img, st);
}

// ---------------------------------------------------------------------------
// Projector: tomography/tv_hpc.F90:137-156.
//   sino(jy,theta) = (1/N) sum_jx bilinear(img; xr, yr)
//   xr = cos(c)*(jx-m) - sin(c)*(jy-m) + m, yr = sin(c)*(jx-m) + cos(c)*(jy-m) + m,
//   c = pi*(theta-90)/180; a sample counts when min(x1,y1) > 1 and
//   max(x1+1,y1+1) < N+1.
// One thread per (bin, angle) ray and slice group, steps in the reference's
// order.  The four bilinear weights are formed once per sample and shared by
// the V slices.
// ---------------------------------------------------------------------------
template <typename Real, int V, bool EX>
__global__ void __launch_bounds__(128) k_radon(const Real* __restrict__ img, const Real* __restrict__ sc,
                                               const float4* __restrict__ xsc, Real* __restrict__ sino, int N,
                                               int T, Real mid, const Real* __restrict__ off)
{
    const int jy = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int t = blockIdx.y * blockDim.y + threadIdx.y;
    const int g = blockIdx.z;
    if (jy > N || t >= T) return;
    // bin jy is read at detector coordinate jy + off[t] (off: per-slice angle offsets, V = 1)
    const ProjRay<Real, EX> ray(sc, xsc, t, jy, mid, off ? off + (size_t)g * T + t : nullptr);
    const Real* u = img + (size_t)g * N * N * V;
    const size_t rowstride = (size_t)N * V;
    Lanes<Real, V> acc;
#pragma unroll
    for (int v = 0; v < V; ++v) acc.v[v] = Real(0);
    for (int jx = 1; jx <= N; ++jx) {
        int x1, y1;
        Real wxl, wxh, wyl, wyh;
        ray.at((Real)jx - mid, x1, y1, wxl, wxh, wyl, wyh);
        if (min(x1, y1) > 1 && max(x1, y1) < N) {
            const Real w11 = wxl * wyl, w21 = wxh * wyl, w12 = wxl * wyh, w22 = wxh * wyh;
            const Real* p = u + ((size_t)(y1 - 1) * N + (x1 - 1)) * V;
            const Lanes<Real, V> a = ld_lanes<Real, V>(p);
            const Lanes<Real, V> b = ld_lanes<Real, V>(p + V);
            const Lanes<Real, V> cc = ld_lanes<Real, V>(p + rowstride);
            const Lanes<Real, V> d = ld_lanes<Real, V>(p + rowstride + V);
#pragma unroll
            for (int v = 0; v < V; ++v)
                acc.v[v] = fma(d.v[v], w22, fma(cc.v[v], w12, fma(b.v[v], w21, fma(a.v[v], w11, acc.v[v]))));
        }
    }
#pragma unroll
    for (int v = 0; v < V; ++v) acc.v[v] = acc.v[v] / (Real)N;
    st_lanes<Real, V>(sino + (((size_t)g * T + t) * N + (jy - 1)) * V, acc);
}

template <typename Real, int V>
void launch_radon(const DevGeom<Real>& g, int G, const Real* img, Real* sino, cudaStream_t st)
{
    dim3 blk(32, 4), grd((g.N + 31) / 32, (g.T + 3) / 4, G);
    if constexpr (sizeof(Real) == 4) {
        if (g.exact) {
            k_radon<Real, V, true><<<grd, blk, 0, st>>>(img, g.sc_fp, g.xsc_fp, sino, g.N, g.T, g.mid, nullptr);
            return;
        }
    }
    k_radon<Real, V, false><<<grd, blk, 0, st>>>(img, g.sc_fp, g.xsc_fp, sino, g.N, g.T, g.mid, nullptr);
}

// ---------------------------------------------------------------------------
// Projector over "pair" images (single precision, 4 slices per thread).
//
// The bilinear sample needs (x1,y1), (x1+1,y1), (x1,y1+1), (x1+1,y1+1).  A
// gather of four separate 16-byte taps per lane makes the L1 data pipe the
// limit (one wavefront per distinct sector).  Here the image is re-laid as
// pairs: P[g][y][x] = (pixel(x,y), pixel(x+1,y)) for the 4 slices, 32 bytes,
// and the transposed PT[g][x][y] = (pixel(x,y), pixel(x,y+1)).  One 256-bit
// load then fetches two taps, and for every angle the kernel reads the copy
// in which the warp's 32 adjacent rays (offset (-sin, cos) per lane) spread
// along the pair axis, so consecutive lanes hit consecutive sectors.
// The arithmetic is identical to k_radon.
// ---------------------------------------------------------------------------
struct __align__(32) Pair4 {
    float a[4];   // first pixel, 4 slices
    float b[4];   // second pixel
};

__device__ __forceinline__ Pair4 ld_pair(const float* p)
{
    Pair4 r;
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(r.a[0]), "=f"(r.a[1]), "=f"(r.a[2]), "=f"(r.a[3]), "=f"(r.b[0]), "=f"(r.b[1]), "=f"(r.b[2]),
          "=f"(r.b[3])
        : "l"(p));
    return r;
}

// Builds P and PT from a lane-layout image (V = 4).  32x32 pixel tiles; the
// transposed copy goes through shared memory so both stores are coalesced.
__global__ void __launch_bounds__(256) k_make_pairs(const float* __restrict__ img, float* __restrict__ P,
                                                    float* __restrict__ PT, int N)
{
    __shared__ float4 tile[33][33];
    const int g = blockIdx.z;
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
    const float4* src = reinterpret_cast<const float4*>(img) + (size_t)g * N * N;
    for (int i = threadIdx.x; i < 33 * 33; i += blockDim.x) {
        const int ty = i / 33, tx = i % 33;
        const int x = x0 + tx, y = y0 + ty;
        tile[ty][tx] = (x < N && y < N) ? src[(size_t)y * N + x] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    float4* Pg = reinterpret_cast<float4*>(P) + (size_t)g * N * N * 2;
    float4* PTg = reinterpret_cast<float4*>(PT) + (size_t)g * N * N * 2;
    for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) {
        const int ty = i / 32, tx = i % 32;
        const int x = x0 + tx, y = y0 + ty;
        if (x < N && y < N) {
            const size_t o = ((size_t)y * N + x) * 2;
            Pg[o] = tile[ty][tx];
            Pg[o + 1] = tile[ty][tx + 1];
        }
        // transposed: row = x, column = y; consecutive threads walk y
        const int xt = x0 + ty, yt = y0 + tx;
        if (xt < N && yt < N) {
            const size_t o = ((size_t)xt * N + yt) * 2;
            PTg[o] = tile[tx][ty];
            PTg[o + 1] = tile[tx + 1][ty];
        }
    }
}

// Staggered rays: a warp holds 32 adjacent rays of one angle and lane b walks
// its own ray in the reference's order jx = 1..N, but started k_b =
// rint(b * cos/sin) steps late (rint(-b * sin/cos) through the transposed
// copy), which puts all 32 samples of an iteration in the same image row (or
// two), 1 to 1.4 pixels apart.  A pair load of the warp then covers one or two
// runs of consecutive pairs, the fewest cache lines 32 distinct samples can
// touch.  Each ray's sum is sequential in jx, as in the reference.
template <bool EX>
__global__ void __launch_bounds__(128) k_radon_pairs(const float* __restrict__ P, const float* __restrict__ PT,
                                                     const float* __restrict__ sc, const float4* __restrict__ xsc,
                                                     const int* __restrict__ order, float* __restrict__ sino, int N,
                                                     int T, float mid)
{
    const int lane = threadIdx.x & 31;
    const int jy = blockIdx.x * 128 + threadIdx.y * 32 + lane + 1;
    const int t = order[blockIdx.y];
    const int g = blockIdx.z;
    const float s = sc[2 * t], c = sc[2 * t + 1];
    const bool transposed = fabsf(c) > fabsf(s);   // uniform across the block
    const float ratio = transposed ? -s / c : c / s;
    const int kb = __float2int_rn((float)lane * ratio);
    const int kend = __float2int_rn(31.f * ratio);
    const int kmin = min(0, kend), kmax = max(0, kend);
    const ProjRay<float, EX> ray(sc, xsc, t, jy, mid, nullptr);
    const float* base = (transposed ? PT : P) + (size_t)g * N * N * 8;
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    for (int i = 1 + kmin; i <= N + kmax; ++i) {
        const int jx = i - kb;
        if (jx < 1 || jx > N || jy > N) continue;
        int x1, y1;
        float wxl, wxh, wyl, wyh;
        ray.at((float)jx - mid, x1, y1, wxl, wxh, wyl, wyh);
        if (min(x1, y1) > 1 && max(x1, y1) < N) {
            const float w11 = wxl * wyl, w21 = wxh * wyl, w12 = wxl * wyh, w22 = wxh * wyh;
            const float* p = transposed ? base + ((size_t)(x1 - 1) * N + (y1 - 1)) * 8
                                        : base + ((size_t)(y1 - 1) * N + (x1 - 1)) * 8;
            const Pair4 r0 = ld_pair(p);
            const Pair4 r1 = ld_pair(p + (size_t)N * 8);
            // normal: r0 = (x1,y1),(x1+1,y1)  r1 = (x1,y1+1),(x1+1,y1+1)
            // transposed: r0 = (x1,y1),(x1,y1+1)  r1 = (x1+1,y1),(x1+1,y1+1)
            const float wb0 = transposed ? w12 : w21;
            const float wa1 = transposed ? w21 : w12;
#pragma unroll
            for (int v = 0; v < 4; ++v)
                acc[v] = fmaf(r1.b[v], w22, fmaf(r1.a[v], wa1, fmaf(r0.b[v], wb0, fmaf(r0.a[v], w11, acc[v]))));
        }
    }
    if (jy <= N) {
        float4 o = make_float4(acc[0] / (float)N, acc[1] / (float)N, acc[2] / (float)N, acc[3] / (float)N);
        *reinterpret_cast<float4*>(sino + (((size_t)g * T + t) * N + (jy - 1)) * 4) = o;
    }
}

// Default variant, without duplication: the lane image itself (16-byte
// pixels) and its transpose, four 128-bit loads per sample, the same staggered
// rays and angle order.  Each copy is N*N*16 bytes per slice group (67 MB at
// N = 2049), half of a pair image, so the copy being read stays resident in
// L2; measured faster than the pair images despite twice the load requests.
__global__ void __launch_bounds__(256) k_make_transpose(const float* __restrict__ img, float* __restrict__ IT, int N)
{
    __shared__ float4 tile[32][33];
    const int g = blockIdx.z;
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
    const float4* src = reinterpret_cast<const float4*>(img) + (size_t)g * N * N;
    float4* dst = reinterpret_cast<float4*>(IT) + (size_t)g * N * N;
    for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) {
        const int ty = i / 32, tx = i % 32;
        if (x0 + tx < N && y0 + ty < N) tile[ty][tx] = src[(size_t)(y0 + ty) * N + x0 + tx];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) {
        const int ty = i / 32, tx = i % 32;   // output row x0+ty, column y0+tx
        if (x0 + ty < N && y0 + tx < N) dst[(size_t)(x0 + ty) * N + y0 + tx] = tile[tx][ty];
    }
}

// One ray of the staggered projector, V slices per pixel (V = 1 or 4), read
// from the copy selected by `transposed` (row = y1 in I, row = x1 in IT).
template <int V, bool EX, bool PAR>
__device__ __forceinline__ void radon_stag_ray(const float* __restrict__ I, const float* __restrict__ IT, int N,
                                               float s, float c, const ProjRay<float, EX>& ray, float mid, int jy,
                                               int lane, bool transposed, float (&acc)[V])
{
    const float ratio = transposed ? -s / c : c / s;
    const int kb = __float2int_rn((float)lane * ratio);
    const int kend = __float2int_rn(31.f * ratio);
    const int kmin = min(0, kend), kmax = max(0, kend);
    const float* base = transposed ? IT : I;
    for (int i = 1 + kmin; i <= N + kmax; ++i) {
        const int jx = i - kb;
        if (jx < 1 || jx > N || jy > N) continue;
        int x1, y1;
        float wxl, wxh, wyl, wyh;
        ray.at((float)jx - mid, x1, y1, wxl, wxh, wyl, wyh);
        if (min(x1, y1) > 1 && max(x1, y1) < N) {
            const float w11 = wxl * wyl, w21 = wxh * wyl, w12 = wxl * wyh, w22 = wxh * wyh;
            const int r0 = transposed ? x1 : y1, c0 = transposed ? y1 : x1;
            const float* p = base + ((size_t)(r0 - 1) * N + (c0 - 1)) * V;
            const float wb = transposed ? w12 : w21, wc = transposed ? w21 : w12;
            if constexpr (PAR) {
                // Rows by parity: the odd row of {r0, r0+1} first, then the
                // even one.  The warp's samples straddle at most two cells
                // (rows R and R+1), so one of the two row loads is the same
                // row for every lane.
                const bool odd = (r0 & 1) != 0;
                const float* pA = odd ? p : p + (size_t)N * V;
                const float* pB = odd ? p + (size_t)N * V : p;
                const float wA0 = odd ? w11 : wc, wA1 = odd ? wb : w22;
                const float wB0 = odd ? wc : w11, wB1 = odd ? w22 : wb;
                const Lanes<float, V> a0 = ld_lanes<float, V>(pA);
                const Lanes<float, V> a1 = ld_lanes<float, V>(pA + V);
                const Lanes<float, V> b0 = ld_lanes<float, V>(pB);
                const Lanes<float, V> b1 = ld_lanes<float, V>(pB + V);
#pragma unroll
                for (int v = 0; v < V; ++v)
                    acc[v] = fmaf(b1.v[v], wB1, fmaf(b0.v[v], wB0, fmaf(a1.v[v], wA1, fmaf(a0.v[v], wA0, acc[v]))));
            } else {
                // a = (r0, c0); b = (r0, c0+1); cc = (r0+1, c0); d = (r0+1, c0+1)
                const Lanes<float, V> a = ld_lanes<float, V>(p);
                const Lanes<float, V> b = ld_lanes<float, V>(p + V);
                const Lanes<float, V> cc = ld_lanes<float, V>(p + (size_t)N * V);
                const Lanes<float, V> d = ld_lanes<float, V>(p + (size_t)N * V + V);
#pragma unroll
                for (int v = 0; v < V; ++v)
                    acc[v] = fmaf(d.v[v], w22, fmaf(cc.v[v], wc, fmaf(b.v[v], wb, fmaf(a.v[v], w11, acc[v]))));
            }
        }
    }
}

// The same ray with the taps of the previous sample kept in registers.  A
// lane's consecutive samples move by (cos, sin) (at most one cell per axis),
// and the rows of the copy advance in one direction per angle (DIR, uniform
// over the block).  When the cell is unchanged no tap is loaded; when only
// the row advanced the shared row is reused and two taps are loaded; any
// other move loads all four.  Values and summation order are those of
// radon_stag_ray<V, EX, false>, so the results are identical.
template <int V, bool EX, int DIR, bool TR, bool F2>
__device__ __forceinline__ void radon_stag_ray_reuse(const float* __restrict__ base, int N, int kb, int i0, int i1,
                                                     const ProjRay<float, EX>& ray, float mid, int jy,
                                                     float (&acc)[V])
{
    constexpr bool transposed = TR;
    int pr = -4, pc = -4;          // cell of the taps held (none yet)
    Lanes<float, V> a, b, cc, d;   // (pr,pc) (pr,pc+1) (pr+1,pc) (pr+1,pc+1)
#pragma unroll
    for (int v = 0; v < V; ++v) a.v[v] = b.v[v] = cc.v[v] = d.v[v] = 0.f;
    const size_t NV = (size_t)N * V;
    for (int i = i0; i <= i1; ++i) {
        const int jx = i - kb;
        if (jx < 1 || jx > N || jy > N) continue;
        int x1, y1;
        float wxl, wxh, wyl, wyh;
        ray.at((float)jx - mid, x1, y1, wxl, wxh, wyl, wyh);
        if (min(x1, y1) > 1 && max(x1, y1) < N) {
            const float w11 = wxl * wyl, w21 = wxh * wyl, w12 = wxl * wyh, w22 = wxh * wyh;
            const int r0 = transposed ? x1 : y1, c0 = transposed ? y1 : x1;
            const float* p = base + ((size_t)(r0 - 1) * N + (c0 - 1)) * V;
            const bool same = (c0 == pc) && (r0 == pr);
            const bool shift = (c0 == pc) && (r0 == pr + DIR);
            if constexpr (DIR > 0) {
                if (shift) {
                    a = cc;
                    b = d;
                }
                if (!same && !shift) {
                    a = ld_lanes<float, V>(p);
                    b = ld_lanes<float, V>(p + V);
                }
                if (!same) {
                    cc = ld_lanes<float, V>(p + NV);
                    d = ld_lanes<float, V>(p + NV + V);
                }
            } else {
                if (shift) {
                    cc = a;
                    d = b;
                }
                if (!same && !shift) {
                    cc = ld_lanes<float, V>(p + NV);
                    d = ld_lanes<float, V>(p + NV + V);
                }
                if (!same) {
                    a = ld_lanes<float, V>(p);
                    b = ld_lanes<float, V>(p + V);
                }
            }
            pr = r0;
            pc = c0;
            const float wb = transposed ? w12 : w21, wc = transposed ? w21 : w12;
            if constexpr (F2 && V % 2 == 0) {
                // the same four FMAs per slice, two slices per instruction
                const float2 W11 = make_float2(w11, w11), WB = make_float2(wb, wb);
                const float2 WC = make_float2(wc, wc), W22 = make_float2(w22, w22);
#pragma unroll
                for (int v = 0; v < V; v += 2) {
                    float2 s2 = make_float2(acc[v], acc[v + 1]);
                    s2 = fma2(make_float2(a.v[v], a.v[v + 1]), W11, s2);
                    s2 = fma2(make_float2(b.v[v], b.v[v + 1]), WB, s2);
                    s2 = fma2(make_float2(cc.v[v], cc.v[v + 1]), WC, s2);
                    s2 = fma2(make_float2(d.v[v], d.v[v + 1]), W22, s2);
                    acc[v] = s2.x;
                    acc[v + 1] = s2.y;
                }
            } else {
#pragma unroll
                for (int v = 0; v < V; ++v)
                    acc[v] = fmaf(d.v[v], w22, fmaf(cc.v[v], wc, fmaf(b.v[v], wb, fmaf(a.v[v], w11, acc[v]))));
            }
        }
    }
}


template <int V, bool EX, bool F2>
__global__ void __launch_bounds__(128) k_radon_stag_reuse(const float* __restrict__ I, const float* __restrict__ IT,
                                                          const float* __restrict__ sc,
                                                          const float4* __restrict__ xsc,
                                                          const int* __restrict__ order, float* __restrict__ sino,
                                                          int N, int T, float mid, bool clip)
{
    const int lane = threadIdx.x & 31;
    const int jy = blockIdx.x * 128 + threadIdx.y * 32 + lane + 1;
    const int t = order[blockIdx.y];
    const int g = blockIdx.z;
    const float s = sc[2 * t], c = sc[2 * t + 1];
    const bool transposed = fabsf(c) > fabsf(s);
    const float ratio = transposed ? -s / c : c / s;
    const int kb = __float2int_rn((float)lane * ratio);
    const int kend = __float2int_rn(31.f * ratio);
    const int kmin = min(0, kend), kmax = max(0, kend);
    const float* base = (transposed ? IT : I) + (size_t)g * N * N * V;
    const ProjRay<float, EX> ray(sc, xsc, t, jy, mid, nullptr);
    float acc[V];
#pragma unroll
    for (int v = 0; v < V; ++v) acc[v] = 0.f;
    // Steps of the warp: the union of its rays' steps that can meet a valid
    // cell (2 <= xr, yr < N), with a margin of two steps; every sample is
    // still tested, so the range only skips samples that fail the test.
    int i0 = 1 + kmin, i1 = N + kmax;
    if (clip) {
        int lo, hi;
        valid_steps(s, c, (float)jy - mid, mid, N, lo, hi);
        if (jy > N || lo > hi) {
            lo = 0x3fffffff;
            hi = -0x3fffffff;
        }
        i0 = max(i0, __reduce_min_sync(0xffffffffu, lo + kb));
        i1 = min(i1, __reduce_max_sync(0xffffffffu, hi + kb));
    }
    // the copy's rows follow y (step sin) in the image, x (step cos) in the transpose
    const bool fwd = (transposed ? c : s) >= 0.f;
    if (transposed) {
        if (fwd) radon_stag_ray_reuse<V, EX, 1, true, F2>(base, N, kb, i0, i1, ray, mid, jy, acc);
        else radon_stag_ray_reuse<V, EX, -1, true, F2>(base, N, kb, i0, i1, ray, mid, jy, acc);
    } else {
        if (fwd) radon_stag_ray_reuse<V, EX, 1, false, F2>(base, N, kb, i0, i1, ray, mid, jy, acc);
        else radon_stag_ray_reuse<V, EX, -1, false, F2>(base, N, kb, i0, i1, ray, mid, jy, acc);
    }
    if (jy <= N) {
        Lanes<float, V> o;
#pragma unroll
        for (int v = 0; v < V; ++v) o.v[v] = acc[v] / (float)N;
        st_lanes<float, V>(sino + (((size_t)g * T + t) * N + (jy - 1)) * V, o);
    }
}

template <int V, bool EX, bool PAR>
__global__ void __launch_bounds__(128) k_radon_stag(const float* __restrict__ I, const float* __restrict__ IT,
                                                    const float* __restrict__ sc, const float4* __restrict__ xsc,
                                                    const int* __restrict__ order, float* __restrict__ sino, int N,
                                                    int T, float mid)
{
    const int lane = threadIdx.x & 31;
    const int jy = blockIdx.x * 128 + threadIdx.y * 32 + lane + 1;
    const int t = order[blockIdx.y];
    const int g = blockIdx.z;
    const float s = sc[2 * t], c = sc[2 * t + 1];
    float acc[V];
#pragma unroll
    for (int v = 0; v < V; ++v) acc[v] = 0.f;
    const ProjRay<float, EX> ray(sc, xsc, t, jy, mid, nullptr);
    radon_stag_ray<V, EX, PAR>(I + (size_t)g * N * N * V, IT + (size_t)g * N * N * V, N, s, c, ray, mid, jy, lane,
                               fabsf(c) > fabsf(s), acc);
    if (jy <= N) {
        Lanes<float, V> o;
#pragma unroll
        for (int v = 0; v < V; ++v) o.v[v] = acc[v] / (float)N;
        st_lanes<float, V>(sino + (((size_t)g * T + t) * N + (jy - 1)) * V, o);
    }
}

// transpose of a lane image, 32 x 32 tiles through shared memory (V = 1 or 4)
template <int V>
__global__ void __launch_bounds__(256) k_transpose_lanes(const float* __restrict__ img, float* __restrict__ IT, int N)
{
    __shared__ Lanes<float, V> tile[32][33];
    const int g = blockIdx.z;
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
    const float* src = img + (size_t)g * N * N * V;
    float* dst = IT + (size_t)g * N * N * V;
    for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) {
        const int ty = i / 32, tx = i % 32;
        if (x0 + tx < N && y0 + ty < N) tile[ty][tx] = ld_lanes_rw<float, V>(src + ((size_t)(y0 + ty) * N + x0 + tx) * V);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) {
        const int ty = i / 32, tx = i % 32;
        if (x0 + ty < N && y0 + tx < N) st_lanes<float, V>(dst + ((size_t)(x0 + ty) * N + y0 + tx) * V, tile[tx][ty]);
    }
}

void launch_radon_v1_fast(const DevGeom<float>& g, int S, const float* img, float* IT, float* sino, cudaStream_t st)
{
    dim3 bp(256), gp((g.N + 31) / 32, (g.N + 31) / 32, S);
    k_transpose_lanes<1><<<gp, bp, 0, st>>>(img, IT, g.N);
    dim3 blk(32, 4), grd((g.N + 127) / 128, g.T, S);
    if (g.exact)
        k_radon_stag<1, true, false><<<grd, blk, 0, st>>>(img, IT, g.sc_fp, g.xsc_fp, g.fp_order, sino, g.N, g.T, g.mid);
    else
        k_radon_stag<1, false, false><<<grd, blk, 0, st>>>(img, IT, g.sc_fp, g.xsc_fp, g.fp_order, sino, g.N, g.T, g.mid);
}

void launch_radon_quads(const DevGeom<float>& g, int G, const float* img, float* IT, float* sino, cudaStream_t st,
                        bool par, bool reuse, bool clip, bool f2)
{
    dim3 bp(256), gp((g.N + 31) / 32, (g.N + 31) / 32, G);
    k_make_transpose<<<gp, bp, 0, st>>>(img, IT, g.N);
    dim3 blk(32, 4), grd((g.N + 127) / 128, g.T, G);
    if (reuse && f2) {
        if (g.exact)
            k_radon_stag_reuse<4, true, true><<<grd, blk, 0, st>>>(img, IT, g.sc_fp, g.xsc_fp, g.fp_order, sino, g.N, g.T,
                                                                   g.mid, clip);
        else
            k_radon_stag_reuse<4, false, true><<<grd, blk, 0, st>>>(img, IT, g.sc_fp, g.xsc_fp, g.fp_order, sino, g.N,
                                                                    g.T, g.mid, clip);
    } else if (reuse) {
        if (g.exact)
            k_radon_stag_reuse<4, true, false><<<grd, blk, 0, st>>>(img, IT, g.sc_fp, g.xsc_fp, g.fp_order, sino, g.N,
                                                                    g.T, g.mid, clip);
        else
            k_radon_stag_reuse<4, false, false><<<grd, blk, 0, st>>>(img, IT, g.sc_fp, g.xsc_fp, g.fp_order, sino, g.N,
                                                                     g.T, g.mid, clip);
    } else if (par) {
        if (g.exact)
            k_radon_stag<4, true, true><<<grd, blk, 0, st>>>(img, IT, g.sc_fp, g.xsc_fp, g.fp_order, sino, g.N, g.T, g.mid);
        else
            k_radon_stag<4, false, true><<<grd, blk, 0, st>>>(img, IT, g.sc_fp, g.xsc_fp, g.fp_order, sino, g.N, g.T, g.mid);
    } else {
        if (g.exact)
            k_radon_stag<4, true, false><<<grd, blk, 0, st>>>(img, IT, g.sc_fp, g.xsc_fp, g.fp_order, sino, g.N, g.T, g.mid);
        else
            k_radon_stag<4, false, false><<<grd, blk, 0, st>>>(img, IT, g.sc_fp, g.xsc_fp, g.fp_order, sino, g.N, g.T, g.mid);
    }
}

void launch_radon_pairs(const DevGeom<float>& g, int G, const float* img, float* P, float* PT, float* sino,
                        cudaStream_t st)
{
    dim3 bp(256), gp((g.N + 31) / 32, (g.N + 31) / 32, G);
    k_make_pairs<<<gp, bp, 0, st>>>(img, P, PT, g.N);
    dim3 blk(32, 4), grd((g.N + 127) / 128, g.T, G);
    if (g.exact)
        k_radon_pairs<true><<<grd, blk, 0, st>>>(P, PT, g.sc_fp, g.xsc_fp, g.fp_order, sino, g.N, g.T, g.mid);
    else
        k_radon_pairs<false><<<grd, blk, 0, st>>>(P, PT, g.sc_fp, g.xsc_fp, g.fp_order, sino, g.N, g.T, g.mid);
}

// ---------------------------------------------------------------------------
// Exact transpose of k_radon, as a gather (no atomics, deterministic).  For
// pixel (px,py) and angle theta the samples that use it as a bilinear tap lie
// within sqrt(2) of its inverse-rotated position; each candidate sample is
// re-evaluated with the projector's own arithmetic, so cells and weights are
// identical to the forward operator's.
// ---------------------------------------------------------------------------
template <typename Real, int V, bool EX>
__global__ void __launch_bounds__(256) k_radon_adjoint(const Real* __restrict__ sino,
                                                       const Real* __restrict__ sc,
                                                       const float4* __restrict__ xsc,
                                                       Real* __restrict__ img, int N, int T, Real mid,
                                                       const Real* __restrict__ off)
{
    const int px = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int py = blockIdx.y * blockDim.y + threadIdx.y + 1;
    const int g = blockIdx.z;
    if (px > N || py > N) return;
    Lanes<Real, V> acc;
#pragma unroll
    for (int v = 0; v < V; ++v) acc.v[v] = Real(0);
    // A pixel on the border is never a tap (taps span 2..N).
    if (px >= 2 && py >= 2) {
        const Real* yg = sino + (size_t)g * T * N * V;
        const Real ex = (Real)px - mid, ey = (Real)py - mid;
        for (int t = 0; t < T; ++t) {
            const Lanes<Real, 2> scp = ld_lanes<Real, 2>(sc + 2 * t);
            const Real s = scp.v[0], c = scp.v[1];
            // tap (px,py) of a sample at (xr,yr) means xr in [px-1,px+1), yr in [py-1,py+1)
            const Real* off_t = off ? off + (size_t)g * T + t : nullptr;
            const Real o = off ? *off_t : Real(0);
            const Real u = c * ex + s * ey + mid;       // jx of the sample at the pixel
            const Real w = -s * ex + c * ey + mid - o;  // jy
            int jx0 = (int)rfloor(u - Real(1.5)), jx1 = (int)rfloor(u + Real(1.5)) + 1;
            int jy0 = (int)rfloor(w - Real(1.5)), jy1 = (int)rfloor(w + Real(1.5)) + 1;
            jx0 = max(jx0, 1); jy0 = max(jy0, 1); jx1 = min(jx1, N); jy1 = min(jy1, N);
            const Real* yt = yg + (size_t)t * N * V;
            for (int jy = jy0; jy <= jy1; ++jy) {
                const ProjRay<Real, EX> ray(sc, xsc, t, jy, mid, off_t);
                Real wsum = Real(0);
                for (int jx = jx0; jx <= jx1; ++jx) {
                    int x1, y1;
                    Real wxl, wxh, wyl, wyh;
                    ray.at((Real)jx - mid, x1, y1, wxl, wxh, wyl, wyh);
                    if (min(x1, y1) > 1 && max(x1, y1) < N && (px == x1 || px == x1 + 1) &&
                        (py == y1 || py == y1 + 1)) {
                        const Real wx = (px == x1) ? wxl : wxh;
                        const Real wy = (py == y1) ? wyl : wyh;
                        wsum += wx * wy;
                    }
                }
                if (wsum != Real(0)) {
                    const Lanes<Real, V> yv = ld_lanes<Real, V>(yt + (size_t)(jy - 1) * V);
#pragma unroll
                    for (int v = 0; v < V; ++v) acc.v[v] = fma(wsum, yv.v[v], acc.v[v]);
                }
            }
        }
    }
#pragma unroll
    for (int v = 0; v < V; ++v) acc.v[v] = acc.v[v] / (Real)N;
    st_lanes<Real, V>(img + ((size_t)g * N * N + (size_t)(py - 1) * N + (px - 1)) * V, acc);
}

template <typename Real, int V>
void launch_radon_adjoint(const DevGeom<Real>& g, int G, const Real* sino, Real* img, cudaStream_t st)
{
    dim3 blk(32, 8), grd((g.N + 31) / 32, (g.N + 7) / 8, G);
    if constexpr (sizeof(Real) == 4) {
        if (g.exact) {
            k_radon_adjoint<Real, V, true><<<grd, blk, 0, st>>>(sino, g.sc_fp, g.xsc_fp, img, g.N, g.T, g.mid, nullptr);
            return;
        }
    }
    k_radon_adjoint<Real, V, false><<<grd, blk, 0, st>>>(sino, g.sc_fp, g.xsc_fp, img, g.N, g.T, g.mid, nullptr);
}

// ---------------------------------------------------------------------------
// Direct ramp filter: tomography/tv_hpc.F90:93-105.
//   out(i,theta) = sum_{j=1..N} sino(j,theta) * filter(i - j + N + 1)
// (every tap lies inside the 2N+1 table).  One block per (angle, group); the
// row and the taps are staged in shared memory; each thread accumulates
// RB consecutive outputs so every row value loaded is used RB times.
// ---------------------------------------------------------------------------
template <typename Real, int V, int RB>
__global__ void __launch_bounds__(256) k_filter_direct(const Real* __restrict__ sino,
                                                       const Real* __restrict__ filt,
                                                       Real* __restrict__ out, int N, int T)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Real* s_x = reinterpret_cast<Real*>(smem_raw);   // N*V
    Real* s_h = s_x + (size_t)N * V;                 // 2N+1
    const int t = blockIdx.x, g = blockIdx.y;
    const Real* row = sino + ((size_t)g * T + t) * N * V;
    for (int i = threadIdx.x; i < N * V; i += blockDim.x) s_x[i] = row[i];
    for (int i = threadIdx.x; i < 2 * N + 1; i += blockDim.x) s_h[i] = filt[i];
    __syncthreads();
    Real* orow = out + ((size_t)g * T + t) * N * V;
    for (int i0 = threadIdx.x * RB; i0 < N; i0 += blockDim.x * RB) {
        Lanes<Real, V> acc[RB];
#pragma unroll
        for (int r = 0; r < RB; ++r)
#pragma unroll
            for (int v = 0; v < V; ++v) acc[r].v[v] = Real(0);
        // output i uses tap index i - j + N (0-based i, j)
        for (int j = 0; j < N; ++j) {
            Lanes<Real, V> x;
#pragma unroll
            for (int v = 0; v < V; ++v) x.v[v] = s_x[(size_t)j * V + v];
#pragma unroll
            for (int r = 0; r < RB; ++r) {
                const Real h = s_h[i0 + r - j + N];
#pragma unroll
                for (int v = 0; v < V; ++v) acc[r].v[v] = fma(x.v[v], h, acc[r].v[v]);
            }
        }
#pragma unroll
        for (int r = 0; r < RB; ++r)
            if (i0 + r < N) st_lanes<Real, V>(orow + (size_t)(i0 + r) * V, acc[r]);
    }
}

template <typename Real, int V>
void launch_filter_direct(const DevGeom<Real>& g, int G, const Real* sino, Real* out, cudaStream_t st)
{
    constexpr int RB = 4;
    size_t sm = sizeof(Real) * ((size_t)g.N * V + 2 * (size_t)g.N + 1 + RB);
    max_dynamic_smem<k_filter_direct<Real, V, RB>>();
    dim3 grd(g.T, G);
    k_filter_direct<Real, V, RB><<<grd, 256, sm, st>>>(sino, g.filt, out, g.N, g.T);
}

// ---- projector with per-angle detector offsets and its derivatives ------------
template <typename Real>
void launch_radon_off(const DevGeom<Real>& g, int S, const Real* img, const Real* off, Real* sino, cudaStream_t st)
{
    dim3 blk(32, 4), grd((g.N + 31) / 32, (g.T + 3) / 4, S);
    if constexpr (sizeof(Real) == 4) {
        if (g.exact) {
            k_radon<Real, 1, true><<<grd, blk, 0, st>>>(img, g.sc_fp, g.xsc_fp, sino, g.N, g.T, g.mid, off);
            return;
        }
    }
    k_radon<Real, 1, false><<<grd, blk, 0, st>>>(img, g.sc_fp, g.xsc_fp, sino, g.N, g.T, g.mid, off);
}
template <typename Real>
void launch_radon_adjoint_off(const DevGeom<Real>& g, int S, const Real* sino, const Real* off, Real* img,
                              cudaStream_t st)
{
    dim3 blk(32, 8), grd((g.N + 31) / 32, (g.N + 7) / 8, S);
    if constexpr (sizeof(Real) == 4) {
        if (g.exact) {
            k_radon_adjoint<Real, 1, true><<<grd, blk, 0, st>>>(sino, g.sc_fp, g.xsc_fp, img, g.N, g.T, g.mid, off);
            return;
        }
    }
    k_radon_adjoint<Real, 1, false><<<grd, blk, 0, st>>>(sino, g.sc_fp, g.xsc_fp, img, g.N, g.T, g.mid, off);
}

// D(jy,theta) = d/d(off) of the projector's value: (1/N) sum_jx of the
// bilinear gradient along the detector direction, dB/dx * (-sin) + dB/dy * cos.
template <typename Real, bool EX>
__global__ void __launch_bounds__(128) k_radon_doff(const Real* __restrict__ img, const Real* __restrict__ sc,
                                                    const float4* __restrict__ xsc, Real* __restrict__ dsino, int N,
                                                    int T, Real mid, const Real* __restrict__ off)
{
    const int jy = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int t = blockIdx.y * blockDim.y + threadIdx.y;
    const int g = blockIdx.z;
    if (jy > N || t >= T) return;
    const Real s = sc[2 * t], c = sc[2 * t + 1];
    const ProjRay<Real, EX> ray(sc, xsc, t, jy, mid, off ? off + (size_t)g * T + t : nullptr);
    const Real* u = img + (size_t)g * N * N;
    Real acc = Real(0);
    for (int jx = 1; jx <= N; ++jx) {
        int x1, y1;
        Real wxl, wxh, wyl, wyh;
        ray.at((Real)jx - mid, x1, y1, wxl, wxh, wyl, wyh);
        if (min(x1, y1) > 1 && max(x1, y1) < N) {
            const Real* p = u + (size_t)(y1 - 1) * N + (x1 - 1);
            const Real a = p[0], b = p[1], cc = p[N], d = p[N + 1];
            const Real gx = (b - a) * wyl + (d - cc) * wyh;
            const Real gy = (cc - a) * wxl + (d - b) * wxh;
            acc += gy * c - gx * s;
        }
    }
    dsino[((size_t)g * T + t) * N + (jy - 1)] = acc / (Real)N;
}
template <typename Real>
void launch_radon_doff(const DevGeom<Real>& g, int S, const Real* img, const Real* off, Real* dsino, cudaStream_t st)
{
    dim3 blk(32, 4), grd((g.N + 31) / 32, (g.T + 3) / 4, S);
    if constexpr (sizeof(Real) == 4) {
        if (g.exact) {
            k_radon_doff<Real, true><<<grd, blk, 0, st>>>(img, g.sc_fp, g.xsc_fp, dsino, g.N, g.T, g.mid, off);
            return;
        }
    }
    k_radon_doff<Real, false><<<grd, blk, 0, st>>>(img, g.sc_fp, g.xsc_fp, dsino, g.N, g.T, g.mid, off);
}
template void launch_radon_off<float>(const DevGeom<float>&, int, const float*, const float*, float*, cudaStream_t);
template void launch_radon_off<double>(const DevGeom<double>&, int, const double*, const double*, double*,
                                       cudaStream_t);
template void launch_radon_adjoint_off<float>(const DevGeom<float>&, int, const float*, const float*, float*,
                                              cudaStream_t);
template void launch_radon_adjoint_off<double>(const DevGeom<double>&, int, const double*, const double*, double*,
                                               cudaStream_t);
template void launch_radon_doff<float>(const DevGeom<float>&, int, const float*, const float*, float*, cudaStream_t);
template void launch_radon_doff<double>(const DevGeom<double>&, int, const double*, const double*, double*,
                                        cudaStream_t);

// ---- explicit instantiations ------------------------------------------------
#define ACU_INST(R, V)                                                                          \
    template void launch_backproject<R, V>(const DevGeom<R>&, int, const R*, R*, cudaStream_t);  \
    template void launch_radon<R, V>(const DevGeom<R>&, int, const R*, R*, cudaStream_t);       \
    template void launch_radon_adjoint<R, V>(const DevGeom<R>&, int, const R*, R*, cudaStream_t); \
    template void launch_filter_direct<R, V>(const DevGeom<R>&, int, const R*, R*, cudaStream_t);
ACU_INST(float, 1)
ACU_INST(float, 4)
ACU_INST(double, 1)
#undef ACU_INST

}  // namespace acu
