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
#include <cmath>
#include <utility>
#include <vector>

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
// selects LINE_ANGLES consecutive entries of `order` (lines_angle_order:
// chunks of neighbouring angles, -1 pads a partial chunk), LINE_NA of them
// walked at once by groups of LINE_WARPS warps over the same rays.  An angle
// with sin >= 0 (rays climbing the rows) walks the bands upward, band `step`;
// the others downward, band nb - 1 - step.
template <bool EX>
__global__ void __launch_bounds__(32 * LINE_WARPS * LINE_NA, 5) k_radon_lines(
    const float* __restrict__ L, float* __restrict__ A, const float* __restrict__ sc, const float4* __restrict__ xsc,
    const int* __restrict__ order, int N, int T, float mid, int step, int H, int nb)
{
    const int lane = threadIdx.x & 31, q = lane >> 3, h = lane & 7;
    const int jy = blockIdx.x * (4 * LINE_WARPS) + (threadIdx.y % LINE_WARPS) * 4 + q + 1;
    const int a0 = threadIdx.y / LINE_WARPS;   // angle slot of this warp's group
    const size_t sg = blockIdx.z;
    const float* p0 = L + sg * N * N * LINE_W + h * 4;
    for (int k = 0; k < LINE_ANGLES / LINE_NA; ++k) {
        const int ti = blockIdx.y * LINE_ANGLES + k * LINE_NA + a0;
        if (jy > N) break;
        const int t = order[ti];
        if (t < 0) continue;
        const float s = sc[2 * t], c = sc[2 * t + 1];
        const int b = s >= 0.f ? step : nb - 1 - step;
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
// (tv_hpc.F90:157).  One thread per 16-byte slot of the sums of super-group
// blockIdx.y, read in order (a warp reads 512 contiguous bytes and writes 64
// contiguous bytes into each of 8 lane groups); groups >= G are padding.
__global__ void k_lines_finish(const float4* __restrict__ A, float4* __restrict__ sino, size_t nsino, int G,
                               float fN)
{
    const size_t sg = blockIdx.y, n = nsino * 8;
    const float4* a_sg = A + sg * n;
    for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < n; j += (size_t)gridDim.x * blockDim.x) {
        const size_t g = sg * 8 + (j & 7);
        if (g >= (size_t)G) continue;
        const float4 a = a_sg[j];
        sino[g * nsino + (j >> 3)] = make_float4(a.x / fN, a.y / fN, a.z / fN, a.w / fN);
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

// Angle order of the band launches, one chunk of LINE_ANGLES consecutive
// angles per block row of the grid (neighbouring angles share pixel lines in
// L1).  A ray whose |sin| is small stays in one band for many steps, so the
// blocks of such angles are the long ones of a band launch (up to N samples
// per ray against about H / |sin| for steep rays).  The chunks are sorted by
// the smallest |sin| they hold, so those blocks are dispatched first and
// never form the launch's last wave, where the SMs would idle waiting for
// them.  The order changes which block computes a ray, not the ray's sum.
std::vector<int> lines_angle_order(const float* sc, int T)
{
    const int nc = (T + LINE_ANGLES - 1) / LINE_ANGLES;
    std::vector<std::pair<float, int>> key(nc);
    for (int ch = 0; ch < nc; ++ch) {
        float m = 2.f;
        for (int t = ch * LINE_ANGLES; t < std::min(T, (ch + 1) * LINE_ANGLES); ++t) m = std::min(m, std::fabs(sc[2 * t]));
        key[ch] = {m, ch};
    }
    std::stable_sort(key.begin(), key.end(),
                     [](const std::pair<float, int>& a, const std::pair<float, int>& b) { return a.first < b.first; });
    std::vector<int> ord((size_t)nc * LINE_ANGLES, -1);
    for (int i = 0; i < nc; ++i)
        for (int k = 0; k < LINE_ANGLES; ++k) {
            const int t = key[i].second * LINE_ANGLES + k;
            if (t < T) ord[(size_t)i * LINE_ANGLES + k] = t;
        }
    return ord;
}

size_t lines_image_floats(int N, int G) { return (size_t)((G + 7) / 8) * N * N * LINE_W; }
size_t lines_sums_floats(int N, int T, int G) { return (size_t)((G + 7) / 8) * T * N * LINE_W; }

void launch_radon_lines(const DevGeom<float>& g, int G, const float* img, float* L, float* A, float* sino,
                        cudaStream_t st)
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
    for (int k = 0; k < nb; ++k) {
        if (g.exact)
            k_radon_lines<true><<<grd, blk, 0, st>>>(L, A, g.sc_fp, g.xsc_fp, g.lines_order, N, T, g.mid, k, H, nb);
        else
            k_radon_lines<false><<<grd, blk, 0, st>>>(L, A, g.sc_fp, g.xsc_fp, g.lines_order, N, T, g.mid, k, H, nb);
    }
    const dim3 fgrd((unsigned)std::min<size_t>((nsino * 8 + 255) / 256, (size_t)152 * 16), SG);
    k_lines_finish<<<fgrd, 256, 0, st>>>(reinterpret_cast<const float4*>(A), reinterpret_cast<float4*>(sino), nsino, G,
                                         (float)N);
}

}  // namespace acu
