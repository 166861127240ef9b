// Projector variant 6: pixel lines (tomography/tv_hpc.F90:129-159).
//
// The batch is regrouped so that one pixel holds 32 consecutive slices, a
// 128-byte line:
//   line image  L[sg][y][x][32]    sg: super-group of 8 lane groups
//   ray sums    A[sg][t][jy][32]
// A warp holds 4 rays of one angle, one per quarter-warp; lane h of a quarter
// carries slices [4h, 4h+4) of its super-group.  Each 128-bit load of a
// quarter-warp therefore reads one aligned 128-byte line, the L1 data path's
// unit, where the staggered kernels' quarters (8 neighbouring rays, 16 bytes
// per pixel) usually straddle two lines.  With the data path relieved, the
// taps are loaded afresh for every sample (no reuse bookkeeping), and a block
// walks two neighbouring angles at once over the same 16 rays: their samples
// meet nearly the same pixel lines, which the second finds in L1.
//
// A super-group's image (N*N*128 bytes, 537 MB at N = 2049) does not fit in
// L2, so the cell rows 2..N-1 are cut into bands of H rows.  Launch k walks,
// for every ray, its samples whose cell row lies in band k (angles with
// sin >= 0, whose rays climb the rows) or band nb-1-k (sin < 0), continuing the
// sum carried in A from the previous launch.  A ray's samples therefore join
// its sum in its own step order jx = 1..N, and the four taps of a sample are
// added in the order of the staggered kernels (|sin| >= |cos|: (x1,y1),
// (x1+1,y1), (x1,y1+1), (x1+1,y1+1); otherwise (x1,y1), (x1,y1+1), (x1+1,y1),
// (x1+1,y1+1)), so the sums are bit-identical to variants 1 to 5.  Two bands
// of H + 1 rows of one super-group are a launch's working set.
#include <algorithm>
#include <atomic>

#include "common.cuh"
#include "kernels.h"

namespace acu {

namespace {

constexpr int LINE_W = 32;        // floats per pixel line: 8 lanes x 4 slices
constexpr int LINE_WARPS = 4;     // warps per angle: 16 rays
constexpr int LINE_NA = 2;        // angles walked at once per block
constexpr int LINE_ANGLES = 4;    // angles per block (LINE_NA at a time)

__device__ __forceinline__ float4 ld_line(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

// acc += a w11 + b wb + c wc + d w22, slice by slice, as fused multiply-adds
// in that order (two slices per instruction).
__device__ __forceinline__ void add_sample(float (&acc)[4], float4 a, float4 b, float4 c, float4 d, float w11,
                                           float wb, float wc, float w22)
{
    const float2 W11 = make_float2(w11, w11), WB = make_float2(wb, wb);
    const float2 WC = make_float2(wc, wc), W22 = make_float2(w22, w22);
    float2 lo = make_float2(acc[0], acc[1]), hi = make_float2(acc[2], acc[3]);
    lo = fma2(make_float2(a.x, a.y), W11, lo);
    hi = fma2(make_float2(a.z, a.w), W11, hi);
    lo = fma2(make_float2(b.x, b.y), WB, lo);
    hi = fma2(make_float2(b.z, b.w), WB, hi);
    lo = fma2(make_float2(c.x, c.y), WC, lo);
    hi = fma2(make_float2(c.z, c.w), WC, hi);
    lo = fma2(make_float2(d.x, d.y), W22, lo);
    hi = fma2(make_float2(d.z, d.w), W22, hi);
    acc[0] = lo.x;
    acc[1] = lo.y;
    acc[2] = hi.x;
    acc[3] = hi.y;
}

// The samples jx = lo..hi of one ray whose cell (x1, y1) is valid and whose
// row y1 lies in [ylo, yhi].  p0: this lane's slices of the super-group's
// line image.  COLS: the ray advances mostly along x (|cos| > |sin|), which
// sets the order of the taps.
template <bool EX, bool COLS>
__device__ __forceinline__ void line_segment(const float* __restrict__ p0, int N, int lo, int hi,
                                             const ProjRay<float, EX>& ray, float mid, int ylo, int yhi,
                                             float (&acc)[4])
{
    const size_t RS = (size_t)N * LINE_W;   // one image row of lines
#pragma unroll 2
    for (int jx = lo; jx <= hi; ++jx) {
        int x1, y1;
        float wxl, wxh, wyl, wyh;
        ray.at((float)jx - mid, x1, y1, wxl, wxh, wyl, wyh);
        if (min(x1, y1) > 1 && max(x1, y1) < N && y1 >= ylo && y1 <= yhi) {
            const float* p = p0 + ((size_t)(y1 - 1) * N + (x1 - 1)) * LINE_W;
            const float4 t00 = ld_line(p), t10 = ld_line(p + LINE_W);
            const float4 t01 = ld_line(p + RS), t11 = ld_line(p + RS + LINE_W);
            const float w11 = wxl * wyl, w21 = wxh * wyl, w12 = wxl * wyh, w22 = wxh * wyh;
            if constexpr (COLS)
                add_sample(acc, t00, t01, t10, t11, w11, w12, w21, w22);
            else
                add_sample(acc, t00, t10, t01, t11, w11, w21, w12, w22);
        }
    }
}

// Narrows the steps [lo, hi] of one ray (bin offset dy) to those whose
// sample can have its cell row in [ylo, yhi]: the real-valued row
// s (jx - m) + c dy + m within one pixel of the band, plus two steps.  A ray
// that hardly climbs (|sin| < 1e-3) keeps its steps when its row range,
// widened by its whole climb, meets the band, and loses them otherwise.
__device__ __forceinline__ void band_steps(float s, float c, float dy, float mid, int N, int ylo, int yhi, int& lo,
                                           int& hi)
{
    const float off = mid + c * dy;   // row at jx = m
    const float y0 = (float)ylo - 1.f, y1 = (float)yhi + 2.f;
    if (fabsf(s) < 1e-3f) {
        const float climb = fabsf(s) * (float)N + 2.f;
        if (off + climb < y0 || off - climb > y1) {
            lo = 1;
            hi = 0;
        }
        return;
    }
    const float t0 = (y0 - off) / s, t1 = (y1 - off) / s;
    lo = max(lo, (int)floorf(fminf(t0, t1) + mid) - 2);
    hi = min(hi, (int)ceilf(fmaxf(t0, t1) + mid) + 2);
}

// Launch `step` of the band walk over super-group blockIdx.z; blockIdx.y
// selects LINE_ANGLES consecutive entries of `order` (the nup angles with
// sin >= 0 first), LINE_NA of them walked at once by groups of LINE_WARPS
// warps over the same rays.
template <bool EX>
__global__ void __launch_bounds__(32 * LINE_WARPS * LINE_NA, 5) k_radon_lines(
    const float* __restrict__ L, float* __restrict__ A, const float* __restrict__ sc, const float4* __restrict__ xsc,
    const int* __restrict__ order, int nup, int N, int T, float mid, int step, int H, int nb)
{
    const int lane = threadIdx.x & 31, q = lane >> 3, h = lane & 7;
    const int jy = blockIdx.x * (4 * LINE_WARPS) + (threadIdx.y % LINE_WARPS) * 4 + q + 1;
    const int a0 = threadIdx.y / LINE_WARPS;   // angle slot of this warp's group
    const size_t sg = blockIdx.z;
    const float* p0 = L + sg * N * N * LINE_W + h * 4;
    for (int k = 0; k < LINE_ANGLES / LINE_NA; ++k) {
        const int ti = blockIdx.y * LINE_ANGLES + k * LINE_NA + a0;
        if (ti >= T || jy > N) break;
        const int t = order[ti];
        const float s = sc[2 * t], c = sc[2 * t + 1];
        const int b = ti < nup ? step : nb - 1 - step;
        const int ylo = 2 + b * H, yhi = min(N - 1, 1 + (b + 1) * H);
        if (ylo > yhi) continue;
        int lo, hi;
        valid_steps(s, c, (float)jy - mid, mid, N, lo, hi);
        band_steps(s, c, (float)jy - mid, mid, N, ylo, yhi, lo, hi);
        if (lo > hi) continue;
        float4* ap = reinterpret_cast<float4*>(A + ((sg * T + t) * N + (jy - 1)) * LINE_W + h * 4);
        const float4 a = *ap;
        float acc[4] = {a.x, a.y, a.z, a.w};
        const ProjRay<float, EX> ray(sc, xsc, t, jy, mid, nullptr);
        if (fabsf(c) > fabsf(s)) line_segment<EX, true>(p0, N, lo, hi, ray, mid, ylo, yhi, acc);
        else line_segment<EX, false>(p0, N, lo, hi, ray, mid, ylo, yhi, acc);
        *ap = make_float4(acc[0], acc[1], acc[2], acc[3]);
    }
}

// ---- variants 9 to 11: the band walk with NA angles per block walked in
// lockstep.  A block holds 16 rays of each of NA consecutive angles (of
// `order`, so neighbouring angles), one quarter-warp per ray as in variant 6.
// Its warps walk the union of their rays' steps in the band in chunks of CH
// steps and meet at a block barrier after each chunk, so at any time the
// block's samples lie in one short stretch of its ray bundles: the pixel lines
// that stretch needs are fetched into L1 once and read by all NA angles.  The
// bundles of neighbouring angles overlap (0.15 degrees apart they diverge by
// ~2.6 px per 1000 px from the centre), so the L2 traffic per sample falls
// roughly as (17 + (NA-1) 2.6 r/1000) / (16 NA).  Samples, taps and order are
// those of variant 6: identical sums.
template <bool EX, int NA, int CH>
__global__ void __launch_bounds__(32 * LINE_WARPS * NA, (NA == 2 ? 5 : NA == 4 ? 2 : 1)) k_radon_lines_lock(
    const float* __restrict__ L, float* __restrict__ A, const float* __restrict__ sc, const float4* __restrict__ xsc,
    const int* __restrict__ order, int nup, int N, int T, float mid, int step, int H, int nb)
{
    __shared__ int rng[2];
    const int lane = threadIdx.x & 31, q = lane >> 3, h = lane & 7;
    const int warp = threadIdx.y;
    const int jy = blockIdx.x * (4 * LINE_WARPS) + (warp % LINE_WARPS) * 4 + q + 1;
    const int slot = warp / LINE_WARPS;
    const size_t sg = blockIdx.z;
    const float* p0 = L + sg * N * N * LINE_W + h * 4;
    const int ti = blockIdx.y * NA + slot;               // warp-uniform
    const bool ok = ti < T && jy <= N;
    const int t = order[ti < T ? ti : T - 1];
    const int jyc = jy <= N ? jy : N;
    const float s = sc[2 * t], c = sc[2 * t + 1];
    const int b = ti < nup ? step : nb - 1 - step;
    const int ylo = 2 + b * H, yhi = min(N - 1, 1 + (b + 1) * H);
    int lo = 1, hi = 0;
    if (ok && ylo <= yhi) {
        valid_steps(s, c, (float)jyc - mid, mid, N, lo, hi);
        band_steps(s, c, (float)jyc - mid, mid, N, ylo, yhi, lo, hi);
    }
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        rng[0] = 0x7fffffff;
        rng[1] = -0x7fffffff;
    }
    __syncthreads();
    if (lo <= hi) {
        atomicMin(&rng[0], lo);
        atomicMax(&rng[1], hi);
    }
    __syncthreads();
    const int J0 = rng[0], J1 = rng[1];
    if (J0 > J1) return;                                 // block-uniform
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    float4* ap = reinterpret_cast<float4*>(A + ((sg * T + t) * N + (jyc - 1)) * LINE_W + h * 4);
    if (lo <= hi) {
        const float4 a = *ap;
        acc[0] = a.x;
        acc[1] = a.y;
        acc[2] = a.z;
        acc[3] = a.w;
    }
    const ProjRay<float, EX> ray(sc, xsc, t, jyc, mid, nullptr);
    const bool cols = fabsf(c) > fabsf(s);
    for (int j = J0; j <= J1; j += CH) {
        const int a = max(lo, j), e = min(hi, j + CH - 1);
        if (cols) line_segment<EX, true>(p0, N, a, e, ray, mid, ylo, yhi, acc);
        else line_segment<EX, false>(p0, N, a, e, ray, mid, ylo, yhi, acc);
        __syncthreads();
    }
    if (lo <= hi) *ap = make_float4(acc[0], acc[1], acc[2], acc[3]);
}

// ---- variant 8: the band walk with each block's pixel lines staged in shared
// memory by the bulk-copy (TMA) engine.  A block is the same 16 rays x 2
// angles as variant 6 (one angle pair per block).  It walks the union of its
// rays' steps in the band in chunks of ST_C steps; for each chunk, the pixel
// lines the chunk's samples can touch lie in the bounding box of the cells of
// its corner samples (positions are affine in (jx, jy)), widened by one line
// and clipped to the grid and the band's rows.  The lanes of warp 0 copy that
// box row by row (each row of the box is one contiguous run of 128-byte lines)
// with cp.async.bulk into one of two shared buffers, completing an mbarrier;
// the next chunk's copies overlap the current chunk's samples.  The line
// loads that miss L1 in variant 6 -- the pace-setter there -- become shared
// memory reads, and the L2 traffic goes through the copy engine instead of
// the L1 miss path.  A tap outside the box (a box too large for the buffer,
// or one wider than the estimate) is read from global memory, so the values
// never depend on the staging; samples, taps and order are those of variant
// 6: identical sums.  Waits are bounded (2^22 polls); a block that gives up
// leaves together, waits (bounded) for its copies in flight and writes NaN
// into its ray sums.
constexpr int ST_C = 8;          // steps per chunk
constexpr int ST_LINES = 432;    // lines per buffer (54 KB)

struct LineStageDesc {
    int bx0, by0, wb, hb;        // box origin (1-based cell coordinates) and size; hb = 0: nothing staged
};

__device__ __forceinline__ unsigned su32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool st_try_wait(unsigned bar, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(bar), "r"(parity)
                 : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool st_wait(unsigned bar, unsigned parity, int limit)
{
    for (int i = 0; i < limit; ++i)
        if (st_try_wait(bar, parity)) return true;
    return false;
}

template <bool EX>
__global__ void __launch_bounds__(32 * LINE_WARPS * LINE_NA, 2) k_radon_lines_staged(
    const float* __restrict__ L, float* __restrict__ A, const float* __restrict__ sc, const float4* __restrict__ xsc,
    const int* __restrict__ order, int nup, int N, int T, float mid, int step, int H, int nb)
{
    extern __shared__ __align__(128) float st_box[];   // [2][ST_LINES][LINE_W]
    __shared__ __align__(8) unsigned long long st_bar[2];
    __shared__ LineStageDesc st_desc[2];
    __shared__ int st_rng[2];                           // block step range: min lo, max hi
    __shared__ int st_band[2 * LINE_NA];                // ylo, yhi of each angle slot
    const int lane = threadIdx.x & 31, q = lane >> 3, h = lane & 7;
    const int warp = threadIdx.y;
    const int jy = blockIdx.x * (4 * LINE_WARPS) + (warp % LINE_WARPS) * 4 + q + 1;
    const int a0 = warp / LINE_WARPS;
    const size_t sg = blockIdx.z;
    const float* Lsg = L + sg * N * N * LINE_W;
    const float* p0 = Lsg + h * 4;
    const size_t RS = (size_t)N * LINE_W;
    const bool ray_ok = jy <= N;
    const int jyc = ray_ok ? jy : N;
    const int ti = blockIdx.y * LINE_NA + a0;           // warp-uniform
    const bool ang_ok = ti < T;
    const int t = order[ang_ok ? ti : T - 1];
    const float s = sc[2 * t], c = sc[2 * t + 1];
    const int b = ti < nup ? step : nb - 1 - step;
    const int ylo = 2 + b * H, yhi = min(N - 1, 1 + (b + 1) * H);
    int lo = 1, hi = 0;
    if (ang_ok && ray_ok && ylo <= yhi) {
        valid_steps(s, c, (float)jyc - mid, mid, N, lo, hi);
        band_steps(s, c, (float)jyc - mid, mid, N, ylo, yhi, lo, hi);
    }
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        st_rng[0] = 0x7fffffff;
        st_rng[1] = -0x7fffffff;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&st_bar[0])) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&st_bar[1])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (threadIdx.x == 0 && (warp % LINE_WARPS) == 0) {
        st_band[2 * a0] = ang_ok ? ylo : 1;
        st_band[2 * a0 + 1] = ang_ok ? yhi : 0;
    }
    __syncthreads();
    if (lo <= hi) {
        atomicMin(&st_rng[0], lo);
        atomicMax(&st_rng[1], hi);
    }
    __syncthreads();
    const int J0 = st_rng[0], J1 = st_rng[1];
    if (J0 > J1) return;                                // block-uniform: no sample in this band
    const int nch = (J1 - J0) / ST_C + 1;
    // the rows the block's taps can use: the union of its angles' bands, plus one
    const int rlo = max(2, min(st_band[0], st_band[2])), rhi = min(N, max(st_band[1], st_band[3]) + 1);

    // warp 0: box of chunk i into buffer i & 1 (lanes 0..7 evaluate the 8
    // corners: angle slot, first/last ray, first/last step)
    auto issue = [&](int i) {
        const int j0 = J0 + i * ST_C, j1 = j0 + ST_C - 1;
        int xmn = 0x7fffffff, xmx = -0x7fffffff, ymn = 0x7fffffff, ymx = -0x7fffffff;
        if (lane < 8) {
            const int sl = lane >> 2;
            const int tic = blockIdx.y * LINE_NA + sl;
            if (tic < T) {
                const int tc = order[tic];
                const int jr = min(N, blockIdx.x * (4 * LINE_WARPS) + ((lane >> 1) & 1) * (4 * LINE_WARPS - 1) + 1);
                const int jxc = (lane & 1) ? j1 : j0;
                const ProjRay<float, EX> ray(sc, xsc, tc, jr, mid, nullptr);
                int x1, y1;
                float a, bb, cc, d;
                ray.at((float)jxc - mid, x1, y1, a, bb, cc, d);
                xmn = x1; xmx = x1; ymn = y1; ymx = y1;
            }
        }
        xmn = __reduce_min_sync(0xffffffffu, xmn);
        xmx = __reduce_max_sync(0xffffffffu, xmx);
        ymn = __reduce_min_sync(0xffffffffu, ymn);
        ymx = __reduce_max_sync(0xffffffffu, ymx);
        const int bx0 = max(1, xmn - 1), bx1 = min(N, xmx + 2);
        const int by0 = max(rlo, ymn - 1), by1 = min(rhi, ymx + 2);
        int wb = bx1 - bx0 + 1, hb = by1 - by0 + 1;
        if (wb <= 0 || hb <= 0 || wb * hb > ST_LINES) hb = 0;
        LineStageDesc& dsc = st_desc[i & 1];
        const unsigned bar = su32(&st_bar[i & 1]);
        if (lane == 0) {
            dsc.bx0 = bx0;
            dsc.by0 = by0;
            dsc.wb = wb;
            dsc.hb = hb;
            const unsigned bytes = hb > 0 ? (unsigned)(wb * hb) * LINE_W * 4u : 0u;
            asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
                             bar),
                         "r"(bytes)
                         : "memory");
        }
        __syncwarp();
        float* dst = st_box + (size_t)(i & 1) * ST_LINES * LINE_W;
        for (int r = lane; r < hb; r += 32) {
            const float* src = Lsg + ((size_t)(by0 + r - 1) * N + (bx0 - 1)) * LINE_W;
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    su32(dst + (size_t)r * wb * LINE_W)),
                "l"(src), "r"((unsigned)wb * LINE_W * 4u), "r"(bar)
                : "memory");
        }
    };
    if (warp == 0) issue(0);

    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    float4* ap = reinterpret_cast<float4*>(A + ((sg * T + t) * N + (jyc - 1)) * LINE_W + h * 4);
    if (lo <= hi) {
        const float4 a = *ap;
        acc[0] = a.x;
        acc[1] = a.y;
        acc[2] = a.z;
        acc[3] = a.w;
    }
    const ProjRay<float, EX> ray(sc, xsc, t, jyc, mid, nullptr);
    const bool cols = fabsf(c) > fabsf(s);
    bool ok = true;
    int i = 0;
    for (; i < nch; ++i) {
        if (warp == 0 && i + 1 < nch) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(i + 1);
        }
        const bool arrived = st_wait(su32(&st_bar[i & 1]), (unsigned)((i >> 1) & 1), 1 << 22);
        if (!__syncthreads_and(arrived)) {
            ok = false;
            break;
        }
        const LineStageDesc dsc = st_desc[i & 1];
        const float* box = st_box + (size_t)(i & 1) * ST_LINES * LINE_W + h * 4;
        const int j0 = max(lo, J0 + i * ST_C), j1 = min(hi, J0 + i * ST_C + ST_C - 1);
#pragma unroll 2
        for (int jx = j0; jx <= j1; ++jx) {
            int x1, y1;
            float wxl, wxh, wyl, wyh;
            ray.at((float)jx - mid, x1, y1, wxl, wxh, wyl, wyh);
            if (min(x1, y1) > 1 && max(x1, y1) < N && y1 >= ylo && y1 <= yhi) {
                const int bx = x1 - dsc.bx0, by = y1 - dsc.by0;
                float4 t00, t10, t01, t11;
                if (bx >= 0 && bx + 1 < dsc.wb && by >= 0 && by + 1 < dsc.hb) {
                    const float* pb = box + (size_t)(by * dsc.wb + bx) * LINE_W;
                    const size_t rs = (size_t)dsc.wb * LINE_W;
                    t00 = *reinterpret_cast<const float4*>(pb);
                    t10 = *reinterpret_cast<const float4*>(pb + LINE_W);
                    t01 = *reinterpret_cast<const float4*>(pb + rs);
                    t11 = *reinterpret_cast<const float4*>(pb + rs + LINE_W);
                } else {
                    const float* pg = p0 + ((size_t)(y1 - 1) * N + (x1 - 1)) * LINE_W;
                    t00 = ld_line(pg);
                    t10 = ld_line(pg + LINE_W);
                    t01 = ld_line(pg + RS);
                    t11 = ld_line(pg + RS + LINE_W);
                }
                const float w11 = wxl * wyl, w21 = wxh * wyl, w12 = wxl * wyh, w22 = wxh * wyh;
                if (cols)
                    add_sample(acc, t00, t01, t10, t11, w11, w12, w21, w22);
                else
                    add_sample(acc, t00, t10, t01, t11, w11, w21, w12, w22);
            }
        }
        __syncthreads();
    }
    if (!ok) {
        // a wait gave up: let the copies already issued land (bounded), then
        // mark this block's ray sums
        for (int r = i; r < min(i + 2, nch); ++r) st_wait(su32(&st_bar[r & 1]), (unsigned)((r >> 1) & 1), 1 << 20);
        const float nan = __int_as_float(0x7fc00000);
        acc[0] = acc[1] = acc[2] = acc[3] = nan;
    }
    if (lo <= hi || !ok)
        if (ray_ok && ang_ok) *ap = make_float4(acc[0], acc[1], acc[2], acc[3]);
}

// Lane image [G][npix][4] -> line image [SG][npix][8][4]; groups G..8SG-1 are
// zero.  One thread per 16-byte slot of the output.
__global__ void k_lines_from_lanes(const float4* __restrict__ img, float4* __restrict__ L, int G, size_t npix,
                                   size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t h = i & 7, pix = (i >> 3) % npix, sg = (i >> 3) / npix;
        const size_t g = sg * 8 + h;
        L[i] = g < (size_t)G ? __ldg(img + g * npix + pix) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// Ray sums [SG][T*N][8][4] -> sinogram in lane layout [G][T*N][4], divided by N
// (tv_hpc.F90:157).  One thread per 16-byte slot of the output.
__global__ void k_lines_finish(const float4* __restrict__ A, float4* __restrict__ sino, size_t nsino, size_t n,
                               float fN)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t g = i / nsino, r = i % nsino;
        const float4 a = A[((g >> 3) * nsino + r) * 8 + (g & 7)];
        sino[i] = make_float4(a.x / fN, a.y / fN, a.z / fN, a.w / fN);
    }
}

unsigned grid_for(size_t n)
{
    const size_t b = (n + 255) / 256;
    return (unsigned)std::min<size_t>(std::max<size_t>(b, 1), (size_t)152 * 64);
}

}  // namespace

int lines_band_rows(int N)
{
    // two bands of H + 1 rows of 128-byte lines in about 64 MB of L2
    const size_t row = (size_t)(N > 0 ? N : 1) * LINE_W * sizeof(float);
    return (int)std::max<size_t>(16, (((size_t)32 << 20) / row) - 1);
}

size_t lines_image_floats(int N, int G) { return (size_t)((G + 7) / 8) * N * N * LINE_W; }
size_t lines_sums_floats(int N, int T, int G) { return (size_t)((G + 7) / 8) * T * N * LINE_W; }

template <int NA, int CH>
static void lock_launch(const DevGeom<float>& g, int SG, const float* L, float* A, int H, int nb, cudaStream_t st)
{
    const int N = g.N, T = g.T;
    dim3 blk(32, LINE_WARPS * NA);
    dim3 grd((N + 4 * LINE_WARPS - 1) / (4 * LINE_WARPS), (T + NA - 1) / NA, SG);
    for (int k = 0; k < nb; ++k) {
        if (g.exact)
            k_radon_lines_lock<true, NA, CH><<<grd, blk, 0, st>>>(L, A, g.sc_fp, g.xsc_fp, g.lines_order, g.lines_nup,
                                                                  N, T, g.mid, k, H, nb);
        else
            k_radon_lines_lock<false, NA, CH><<<grd, blk, 0, st>>>(L, A, g.sc_fp, g.xsc_fp, g.lines_order,
                                                                   g.lines_nup, N, T, g.mid, k, H, nb);
    }
}

void launch_radon_lines(const DevGeom<float>& g, int G, const float* img, float* L, float* A, float* sino,
                        cudaStream_t st, int mode)
{
    const int N = g.N, T = g.T, SG = (G + 7) / 8;
    if (G <= 0 || N <= 0 || T <= 0) return;
    const size_t npix = (size_t)N * N, nsino = (size_t)T * N;
    const size_t nl = (size_t)SG * npix * 8;
    k_lines_from_lanes<<<grid_for(nl), 256, 0, st>>>(reinterpret_cast<const float4*>(img),
                                                     reinterpret_cast<float4*>(L), G, npix, nl);
    cudaMemsetAsync(A, 0, sizeof(float) * lines_sums_floats(N, T, G), st);
    const int H = lines_band_rows(N), nb = std::max(1, (N - 2 + H - 1) / H);
    dim3 blk(32, LINE_WARPS * LINE_NA);
    dim3 grd((N + 4 * LINE_WARPS - 1) / (4 * LINE_WARPS), (T + LINE_ANGLES - 1) / LINE_ANGLES, SG);
    const bool staged = mode == 1;
    if (mode == 2) lock_launch<2, 16>(g, SG, L, A, H, nb, st);
    if (mode == 3) lock_launch<4, 16>(g, SG, L, A, H, nb, st);
    if (mode == 4) lock_launch<8, 16>(g, SG, L, A, H, nb, st);
    if (staged) {
        // the two buffers (108 KB) need the opt-in above the default 48 KB;
        // the attribute counts only dynamic shared memory, and together with
        // the kernel's static barriers it must stay within the 227 KB limit
        const size_t smem = sizeof(float) * 2 * ST_LINES * LINE_W;
        static std::atomic<unsigned long long> set{0};   // per device, once
        int dev = 0;
        cudaGetDevice(&dev);
        const unsigned long long bit = 1ull << (dev & 63);
        if (!(set.load(std::memory_order_acquire) & bit)) {
            cudaFuncSetAttribute(k_radon_lines_staged<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            cudaFuncSetAttribute(k_radon_lines_staged<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            set.fetch_or(bit, std::memory_order_release);
        }
        dim3 sgrd((N + 4 * LINE_WARPS - 1) / (4 * LINE_WARPS), (T + LINE_NA - 1) / LINE_NA, SG);
        for (int k = 0; k < nb; ++k) {
            if (g.exact)
                k_radon_lines_staged<true><<<sgrd, blk, smem, st>>>(L, A, g.sc_fp, g.xsc_fp, g.lines_order,
                                                                     g.lines_nup, N, T, g.mid, k, H, nb);
            else
                k_radon_lines_staged<false><<<sgrd, blk, smem, st>>>(L, A, g.sc_fp, g.xsc_fp, g.lines_order,
                                                                      g.lines_nup, N, T, g.mid, k, H, nb);
        }
    }
    for (int k = 0; k < (mode != 0 ? 0 : nb); ++k) {
        if (g.exact)
            k_radon_lines<true><<<grd, blk, 0, st>>>(L, A, g.sc_fp, g.xsc_fp, g.lines_order, g.lines_nup, N, T, g.mid,
                                                      k, H, nb);
        else
            k_radon_lines<false><<<grd, blk, 0, st>>>(L, A, g.sc_fp, g.xsc_fp, g.lines_order, g.lines_nup, N, T,
                                                       g.mid, k, H, nb);
    }
    const size_t no = (size_t)G * nsino;
    k_lines_finish<<<grid_for(no), 256, 0, st>>>(reinterpret_cast<const float4*>(A), reinterpret_cast<float4*>(sino),
                                                 nsino, no, (float)N);
}

}  // namespace acu
