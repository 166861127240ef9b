// Internal launcher declarations shared by the .cu translation units.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <vector>

namespace acu {

// The exact backprojection's per-angle table as a kernel parameter (up to
// BP_TMAX angles; kernel parameters may take up to 32 KB).
constexpr int BP_TMAX = 1920;
struct BpTable {
    float4 v[BP_TMAX];
};

// Geometry of one reconstruction grid on the device, for one precision.
// All tables are computed on the host (tables.cpp) with the reference's
// arithmetic and uploaded once.
template <typename Real>
struct DevGeom {
    int N = 0, T = 0;
    Real mid = 0;                 // (N+1)/2, integer division (tv_hpc.F90:15)
    const Real* sc_bp = nullptr;  // [T][2] sin, cos of pi*(90-theta)/180
    const Real* sc_fp = nullptr;  // [T][2] sin, cos of pi*(theta-90)/180
    const Real* filt = nullptr;   // [2N+1] filter taps (tv_hpc.F90:53-56)
    const Real* cmask = nullptr;  // [N][N] tapered mask times pi/T (tv_hpc.F90:58-74)
    const Real* fft_h = nullptr;  // [L] real spectrum of the wrapped filter
    const Real* fft_h_x = nullptr;  // [L] the same from FP64 taps, used with exact positions
    const float2* fft_tw16 = nullptr;  // L = 4096, single precision: radix-16 pass twiddles (tables.h)
    const float2* fft_tw = nullptr; // [L/2] twiddles exp(-2 pi i k / L) (float)
    const double2* fft_tw64 = nullptr;
    int fft_L = 0, fft_log2L = 0;
    const int* fp_order = nullptr;  // [T] projector angles, |sin| >= |cos| first
    const int* lines_order = nullptr;  // projector variant 6: lines_angle_order (chunks of angles, -1 padded)
    // exact positions (single precision only): split FP64 angle tables,
    // [T] x (s_a, c_a, s_r, c_r); exact != 0 selects them
    const float4* xsc_bp = nullptr;
    const float4* xsc_fp = nullptr;
    int exact = 0;
    const float4* h_xsc_bp = nullptr;   // host copy of xsc_bp (for the parameter table)
    const float4* h_sc_bp = nullptr;    // host copy of sc_bp as (sin, cos, 0, 0), single precision
    int bp_param = 1;                   // backprojection: angle table in the launch parameters when T <= BP_TMAX
    int bp_groups = 0;   // slice groups per backprojection thread: 0 auto (1 with the parameter table, else 2), 1, 2 or 4
    int bp_tma = 0;      // 1: exact backprojection from sinogram bins staged in shared memory by bulk copies
};

// ---- radon operators (kernels_radon.cu); arrays in lane layout ------------
template <typename Real, int V>
void launch_backproject(const DevGeom<Real>& g, int G, const Real* q, Real* img, cudaStream_t st);
template <typename Real, int V>
void launch_radon(const DevGeom<Real>& g, int G, const Real* img, Real* sino, cudaStream_t st);
// Projector through pair images (float, 4 slices per thread): P and PT are
// work buffers of 2 * N * N * 4 floats per slice group each.
void launch_radon_pairs(const DevGeom<float>& g, int G, const float* img, float* P, float* PT, float* sino,
                        cudaStream_t st);
// Same projector on the lane image and its transpose IT (N * N * 4 floats per
// slice group), four 128-bit loads per sample.
// par: the four taps loaded by row parity (odd row of the cell first);
// reuse: taps of the previous sample kept in registers; clip (with reuse):
// steps limited to those that can meet a valid cell.
void launch_radon_quads(const DevGeom<float>& g, int G, const float* img, float* IT, float* sino, cudaStream_t st,
                        bool par = false, bool reuse = false, bool clip = false, bool f2 = false);
// Projector variant 6 (kernels_lines.cu): the batch regrouped into 128-byte
// pixel lines of 32 slices, walked in bands of rows that stay in L2.  L and A
// are work buffers of lines_image_floats and lines_sums_floats floats.
void launch_radon_lines(const DevGeom<float>& g, int G, const float* img, float* L, float* A, float* sino,
                        cudaStream_t st);
size_t lines_image_floats(int N, int G);
size_t lines_sums_floats(int N, int T, int G);
int lines_band_rows(int N);
// The band launches' angle order for single-precision (sin, cos) pairs sc[2T].
std::vector<int> lines_angle_order(const float* sc, int T);
// The staggered projector for one slice per thread (plain layout); IT is a
// work buffer of N * N floats per slice.
void launch_radon_v1_fast(const DevGeom<float>& g, int S, const float* img, float* IT, float* sino, cudaStream_t st);
template <typename Real, int V>
void launch_radon_adjoint(const DevGeom<Real>& g, int G, const Real* sino, Real* img, cudaStream_t st);
template <typename Real, int V>
void launch_filter_direct(const DevGeom<Real>& g, int G, const Real* sino, Real* out, cudaStream_t st);
template <typename Real, int V>
void launch_filter_fft(const DevGeom<Real>& g, int G, const Real* sino, Real* out, cudaStream_t st);
template <typename Real>
bool fft_fits(int L);

// ---- projector / adjoint with per-slice, per-angle detector offsets off[S][T]
// (plain layout, one slice per thread) and the offset derivative of the
// projector (kernels_radon.cu); the loss / gradient steps (kernels_grad.cu).
template <typename Real>
void launch_radon_off(const DevGeom<Real>& g, int S, const Real* img, const Real* off, Real* sino, cudaStream_t st);
template <typename Real>
void launch_radon_adjoint_off(const DevGeom<Real>& g, int S, const Real* sino, const Real* off, Real* img,
                              cudaStream_t st);
template <typename Real>
void launch_radon_doff(const DevGeom<Real>& g, int S, const Real* img, const Real* off, Real* dsino, cudaStream_t st);
template <typename Real>
struct GradEw {
    // r = A u - y in place (r holds A u), per-slice FP64 partials of 1/2 |r|^2
    static void residual(size_t n_per, int S, Real* r, const Real* y, double* part, int nblk, cudaStream_t st);
    // grad_u += lambda * dTV_eps/du; per-slice partials of lambda * TV_eps(u)
    static void tv_grad(int N, int S, Real lambda, Real eps, const Real* u, Real* grad, double* part, int nblk,
                        cudaStream_t st);
    // grad_off[s][t] = sum_jy r * D
    static void off_grad(int N, int T, int S, const Real* r, const Real* D, Real* grad_off, cudaStream_t st);
};
void launch_sum_rows(const double* part, int rows, int nblk, double* out, cudaStream_t st);

// ---- layout conversion (kernels_tv.cu) ------------------------------------
// plain [S][npos] <-> lanes [G][npos][V]; slices >= S of the last group are 0.
template <typename Real, int V>
void launch_to_lanes(const Real* plain, Real* lanes, int S, size_t npos, cudaStream_t st);
template <typename Real, int V>
void launch_from_lanes(const Real* lanes, Real* plain, int S, size_t npos, cudaStream_t st);
template <typename Real>
void launch_convert(const float* in, Real* out, size_t n, cudaStream_t st);

// ---- split-Bregman / CG elementwise steps (kernels_tv.cu) ----------------
// All images are [G][N][N][V]; per-slice scalars are double[G*V].
struct TvScalars {
    double* rsold;   // [S]
    double* alpha;   // [S]
    double* beta;    // [S]
    double* delta;   // [S] Err_diff
    double* part;    // [nblk_max * S] block partial sums
    int nblk;        // blocks of the elementwise grid
};

template <typename Real, int V>
struct TvEw {
    // ifkt2 (optional) is added to ifkt
    static void rhs(int N, int G, Real mu, Real lambda, const Real* ifkt, const Real* dx,
                    const Real* bx, const Real* dy, const Real* by, Real* rhs, cudaStream_t st,
                    const Real* ifkt2 = nullptr);
    static void resid(int N, int G, Real mu, Real lambda, const Real* rhs, const Real* iukt,
                      const Real* uk, Real* r, Real* p, const TvScalars& sc, cudaStream_t st);
    static void apply(int N, int G, Real mu, Real lambda, const Real* irpt, const Real* p,
                      Real* Ap, const TvScalars& sc, cudaStream_t st);
    // with irpt and bd: bd -= alpha irpt as well (the carried iradon(f - radon(uk)))
    static void update(int N, int G, const Real* p, const Real* Ap, Real* uk, Real* r,
                       const TvScalars& sc, cudaStream_t st, const Real* irpt = nullptr, Real* bd = nullptr);
    static void pupdate(int N, int G, const Real* r, Real* p, const TvScalars& sc, cudaStream_t st);
    static void shrink(int N, int G, Real lambda, const Real* uk, Real* dx, Real* bx, Real* dy,
                       Real* by, const Real* ukp, const TvScalars& sc, cudaStream_t st);
    static void fk_update(size_t n, Real* fk, const Real* f, const Real* ruk, cudaStream_t st);
    // y += alpha_slice * x over sinograms (radon(uk) carried through uk += alpha p)
    static void sino_axpy(int T, int N, int G, const Real* x, Real* y, const TvScalars& sc, cudaStream_t st);
    // out = a - b (the data residual fk - radon(uk) of the merged initial residual)
    static void diff(size_t n, const Real* a, const Real* b, Real* out, cudaStream_t st);
    // y += x
    static void add(size_t n, const Real* x, Real* y, cudaStream_t st);
};

// Finalisers of the FP64 CG scalars (one block per slice, fixed order).
// which: 0 -> rsold = sum;  1 -> alpha = rsold / sum;  2 -> beta = sum / rsold,
// rsold = sum;  3 -> delta = sum.
void launch_cg_finalize(int which, int S, const TvScalars& sc, cudaStream_t st);

}  // namespace acu
