/*
 * acumen_oracle -- CPU restatement of the Acumen tomography hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py load this library, and only as
 * the checker or the timed CPU baseline.  The product (libacumen_gpu.so)
 * never links or calls it.
 *
 * The reference (ornlneutronimaging/acumen) is Fortran-90 + OpenACC and
 * cannot be compiled in this image (no Fortran compiler, no MPI), and it
 * ships no tests or golden vectors, so this restatement is pinned by
 * analytic known answers (tests/test_oracle.py) instead: parity unpinned
 * against the reference's own outputs.
 *
 * Two instantiations of oracle_impl.h:
 *   *_f32  single precision, source operation order, no FMA contraction
 *          (built with -ffp-contract=off), libm sinf/cosf/expf/logf;
 *   *_f64  the same loops in double precision (the FP64 oracle).
 * The remaining functions restate the projection-to-sinogram steps in the
 * reference's single precision.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define R(x) ((REAL)(x))

/* ---------------- single precision ---------------- */
#define REAL float
#define SFX(n) n##_f32
#define RATAN atanf
#define RSIN sinf
#define RCOS cosf
#define RE expf
#define RSQRT sqrtf
#define RFLOOR floorf
#define RMAX fmaxf
#define RABS fabsf
#include "oracle_impl.h"
#undef REAL
#undef SFX
#undef RATAN
#undef RSIN
#undef RCOS
#undef RE
#undef RSQRT
#undef RFLOOR
#undef RMAX
#undef RABS

/* ---------------- double precision ---------------- */
#define REAL double
#define SFX(n) n##_f64
#define RATAN atan
#define RSIN sin
#define RCOS cos
#define RE exp
#define RSQRT sqrt
#define RFLOOR floor
#define RMAX fmax
#define RABS fabs
#include "oracle_impl.h"
#undef REAL
#undef SFX

/* ====================================================================== */
/* Projection preprocessing (single precision, as the reference)          */
/* ====================================================================== */

/* tomography/fits_to_hpc.F90:183-194 / 196-210 -- average of a frame stack:
 * running single-precision sum in frame order, then divided by the count. */
void orc_frame_average(int nframes, long npix, const float *frames, float *out)
{
    for (long i = 0; i < npix; ++i) out[i] = 0.0f;
    for (int j = 0; j < nframes; ++j)
        for (long i = 0; i < npix; ++i) out[i] = out[i] + frames[(size_t)j * npix + i];
    for (long i = 0; i < npix; ++i) out[i] = out[i] / (float)nframes;
}

/* tomography/fits_to_hpc.F90:243 (mode 0) and the flat/dark form of :244
 * (mode 1) -- log-normalisation of one projection.                        */
void orc_normalize(int mode, long npix, const float *img, const float *ob,
                   const float *df, float *out)
{
    const float eps = 1e-16f;
    for (long i = 0; i < npix; ++i) {
        if (mode == 0) {
            out[i] = -logf(img[i] / fmaxf(ob[i], 1.0f));
        } else {
            out[i] = -logf(fmaxf(img[i] - df[i], eps) / fmaxf(ob[i] - df[i], 1.0f));
        }
    }
}

/* tomography/tv_hpc.F90:546-547 -- first index (1-based) of the minimum of
 * |theta - target|, as Fortran MINLOC.                                    */
int orc_minloc_abs(int n, const float *theta, float target)
{
    int best = 1;
    float bv = fabsf(theta[0] - target);
    for (int j = 2; j <= n; ++j) {
        float v = fabsf(theta[j - 1] - target);
        if (v < bv) { bv = v; best = j; }
    }
    return best;
}

/* tomography/projections_to_sinogram_hpc.F90:141-224 -- the projection at
 * exactly `target` degrees (0 or 180): the nearest projection when its angle
 * equals the target or it has no neighbour on the far side, else a linear
 * interpolation between the two projections that bracket it.
 * proj: nfiles projections of npix floats each.                            */
void orc_pick_angle(int nfiles, const float *theta, long npix, const float *proj,
                    float target, float *out)
{
    int js = orc_minloc_abs(nfiles, theta, target);
    const float *pa, *pb;
    float ta, tb;
    if (theta[js - 1] == target) {
        memcpy(out, proj + (size_t)(js - 1) * npix, sizeof(float) * npix);
        return;
    }
    if (theta[js - 1] <= target) {
        if (js < nfiles) {
            pa = proj + (size_t)(js - 1) * npix; pb = proj + (size_t)js * npix;
            ta = theta[js - 1]; tb = theta[js];
        } else {
            memcpy(out, proj + (size_t)(js - 1) * npix, sizeof(float) * npix);
            return;
        }
    } else {
        if (js > 1) {
            pa = proj + (size_t)(js - 2) * npix; pb = proj + (size_t)(js - 1) * npix;
            ta = theta[js - 2]; tb = theta[js - 1];
        } else {
            memcpy(out, proj + (size_t)(js - 1) * npix, sizeof(float) * npix);
            return;
        }
    }
    for (long i = 0; i < npix; ++i)
        out[i] = (((target - ta) * (pb[i] - pa[i])) / (tb - ta)) + pa[i];
}

/* Bilinear resample of one (ndet x nrows) projection onto the padded
 * (ndet+add) x nrows grid under rotation theta and shift (fraction of ndet),
 * with the clamps of tomography/projections_to_sinogram_hpc.F90:456-470.
 * cth/sth are cos/sin of theta computed by the caller.                     */
static inline float resample_at(int ndet, int nrows, int add, const float *src,
                                float cth, float sth, float shift, int jx, int jy)
{
    const float mx = (float)(ndet + add - 1) / 2.0f;
    const float my = (float)(nrows - 1) / 2.0f;
    const float ss = (float)ndet;
    float ax = ((float)jx - mx) - ss * shift;
    float ay = (float)jy - my;
    float xr = fminf(fmaxf((cth * ax - sth * ay) + mx, 1.0f), (float)ndet);
    float yr = fminf(fmaxf((sth * ax + cth * ay) + my, 1.0f), (float)nrows);
    int y1 = (int)floorf(yr); y1 = y1 < 1 ? 1 : (y1 > nrows ? nrows : y1);
    int y2 = y1 + 1; y2 = y2 < 1 ? 1 : (y2 > nrows ? nrows : y2);
    int x1 = (int)floorf(xr); x1 = x1 < 1 ? 1 : (x1 > ndet ? ndet : x1);
    int x2 = x1 + 1; x2 = x2 < 1 ? 1 : (x2 > ndet ? ndet : x2);
#define S_(x, y) src[(size_t)((y) - 1) * ndet + ((x) - 1)]
    float wxl = (float)x2 - xr, wxh = xr - (float)x1;
    float wyl = (float)y2 - yr, wyh = yr - (float)y1;
    return (((S_(x1, y1) * wxl) * wyl + (S_(x2, y1) * wxh) * wyl) + (S_(x1, y2) * wxl) * wyh)
           + (S_(x2, y2) * wxh) * wyh;
#undef S_
}

void orc_resample(int ndet, int nrows, const float *src, float theta, float shift, float *out)
{
    int add = (ndet % 2 == 0) ? 1 : 0;
    float c = cosf(theta), s = sinf(theta);
    for (int jy = 1; jy <= nrows; ++jy)
        for (int jx = 1; jx <= ndet + add; ++jx)
            out[(size_t)(jy - 1) * (ndet + add) + (jx - 1)] =
                resample_at(ndet, nrows, add, src, c, s, shift, jx, jy);
}

/* Mirror mismatch sum_{jx,jy} |V0(jx,jy) - V180(ndet+add-jx+1,jy)| of the two
 * resampled projections, loop order jx outer, jy inner
 * (projections_to_sinogram_hpc.F90:279-284).  red_mode 0: single-precision
 * running sum as the reference; 1: double accumulation.                   */
static double mirror_error(int ndet, int nrows, const float *p0, const float *p180,
                           float theta, float shift, int red_mode)
{
    int add = (ndet % 2 == 0) ? 1 : 0;
    int nx = ndet + add;
    float c = cosf(theta), s = sinf(theta);
    float *v0 = (float *)malloc(sizeof(float) * (size_t)nx * nrows);
    float *v1 = (float *)malloc(sizeof(float) * (size_t)nx * nrows);
    for (int jy = 1; jy <= nrows; ++jy)
        for (int jx = 1; jx <= nx; ++jx) {
            v0[(size_t)(jy - 1) * nx + jx - 1] = resample_at(ndet, nrows, add, p0, c, s, shift, jx, jy);
            v1[(size_t)(jy - 1) * nx + jx - 1] = resample_at(ndet, nrows, add, p180, c, s, shift, jx, jy);
        }
    double e64 = 0.0;
    float e32 = 0.0f;
    for (int jx = 1; jx <= nx; ++jx)
        for (int jy = 1; jy <= nrows; ++jy) {
            float d = fabsf(v0[(size_t)(jy - 1) * nx + jx - 1] - v1[(size_t)(jy - 1) * nx + (nx - jx)]);
            if (red_mode == 0) e32 = e32 + d; else e64 += d;
        }
    free(v0); free(v1);
    return red_mode == 0 ? (double)e32 : e64;
}

/* tomography/projections_to_sinogram_hpc.F90:231-364 -- rotation-axis
 * registration: centre-of-mass initial shift, then a multiplicative pattern
 * search over (tilt, shift).  Outputs theta [rad] and shift [fraction of
 * ndet].  evals (optional) receives the number of objective evaluations.  */
void orc_register(int ndet, int nrows, const float *p0, const float *p180, int red_mode,
                  float *best_theta_out, float *best_shift_out, int *evals)
{
    int add = (ndet % 2 == 0) ? 1 : 0;
    float tm = 0.0f, cmx0 = 0.0f, cmx180 = 0.0f;
    double tm64 = 0.0, c064 = 0.0, c18064 = 0.0;
    for (int jx = 1; jx <= ndet; ++jx)
        for (int jy = 1; jy <= nrows; ++jy) {
            float a = p0[(size_t)(jy - 1) * ndet + jx - 1];
            float b = p180[(size_t)(jy - 1) * ndet + jx - 1];
            float w = ((2.0f * (float)(ndet + add)) * (float)(jx - 1)) / (float)(ndet + add - 1)
                      - (float)ndet - (float)add;
            if (red_mode == 0) {
                tm = (tm + a) + b;
                cmx0 = cmx0 + a * w;
                cmx180 = cmx180 + b * w;
            } else {
                tm64 = (tm64 + a) + b;
                c064 += (double)(a * w);
                c18064 += (double)(b * w);
            }
        }
    if (red_mode != 0) { tm = (float)tm64; cmx0 = (float)c064; cmx180 = (float)c18064; }
    const float shift_scale = (float)ndet;
    float best_shift = -((cmx0 / tm + cmx180 / tm) / (2.0f * shift_scale));
    float best_theta = 0.0f;
    float dshift = 1e-4f, dtheta = 1e-4f;
    const int n_sp = 6;
    const float n_mag = 1.05f, n_min = 2.0f / (float)n_sp;
    int ne = 1;
    float best_error = (float)mirror_error(ndet, nrows, p0, p180, best_theta, best_shift, red_mode);
    while (fmaxf(dtheta, dshift) > 1e-8f) {
        float perr = best_error;
        for (int jsp = 1; jsp <= n_sp; ++jsp) {
            float th = best_theta + dtheta * (float)(jsp - n_sp / 2);
            float e = (float)mirror_error(ndet, nrows, p0, p180, th, best_shift, red_mode);
            ++ne;
            if (e < best_error) { best_theta = th; best_error = e; }
        }
        dtheta = (best_error < perr) ? n_mag * dtheta : n_min * dtheta;
        perr = best_error;
        for (int jsp = 1; jsp <= n_sp; ++jsp) {
            float sh = best_shift + dshift * (float)(jsp - n_sp / 2);
            float e = (float)mirror_error(ndet, nrows, p0, p180, best_theta, sh, red_mode);
            ++ne;
            if (e < best_error) { best_shift = sh; best_error = e; }
        }
        dshift = (best_error < perr) ? n_mag * dshift : n_min * dshift;
        if (ne > 200000) break;
    }
    *best_theta_out = best_theta;
    *best_shift_out = best_shift;
    if (evals) *evals = ne;
}

/* tomography/projections_to_sinogram_hpc.F90:426-452 -- median of the 3x3
 * spatial x 3 projection box with clamped edges, by the reference's exchange
 * sort (descending) taking element 14 of 27.  The reference's slot index
 * 3*(jxs+1-1)+jys+2 writes slots -2..24; this restatement uses the intended
 * slots 1..27 (3*(jxs+1)+(jys+1)+1, then +9, +18).                        */
void orc_median27(int ndet, int nrows, const float *dl, const float *dc, const float *dr, float *out)
{
    for (int jy = 1; jy <= nrows; ++jy)
        for (int jx = 1; jx <= ndet; ++jx) {
            float reg[27];
            for (int jxs = -1; jxs <= 1; ++jxs)
                for (int jys = -1; jys <= 1; ++jys) {
                    int cjx = jx + jxs; cjx = cjx < 1 ? 1 : (cjx > ndet ? ndet : cjx);
                    int cjy = jy + jys; cjy = cjy < 1 ? 1 : (cjy > nrows ? nrows : cjy);
                    int slot = 3 * (jxs + 1) + (jys + 1);
                    size_t o = (size_t)(cjy - 1) * ndet + (cjx - 1);
                    reg[slot] = dl[o];
                    reg[slot + 9] = dc[o];
                    reg[slot + 18] = dr[o];
                }
            for (int i = 0; i < 26; ++i) {
                float ra = reg[i];
                for (int j = i + 1; j < 27; ++j) {
                    float rb = reg[j];
                    if (rb > ra) { reg[j] = ra; reg[i] = rb; ra = rb; }
                }
            }
            out[(size_t)(jy - 1) * ndet + (jx - 1)] = reg[13];
        }
}

/* tomography/projections_to_sinogram_hpc.F90:397-487 -- one projection job:
 * median over (previous, this, next) projections, resample, and transpose
 * row jy into sinogram jy at angle index job (0-based).
 * proj: nfiles normalised projections (ndet x nrows each);
 * sino: nrows sinograms of nfiles x (ndet+add) floats.                     */
void orc_proj_to_sino(int nfiles, int ndet, int nrows, const float *proj, float theta,
                      float shift, float *sino)
{
    int add = (ndet % 2 == 0) ? 1 : 0;
    int nx = ndet + add;
    size_t npix = (size_t)ndet * nrows;
    float *med = (float *)malloc(sizeof(float) * npix);
    float *res = (float *)malloc(sizeof(float) * (size_t)nx * nrows);
    for (int job = 0; job < nfiles; ++job) {
        const float *dc = proj + (size_t)job * npix;
        const float *dl = job > 0 ? dc - npix : dc;
        const float *dr = job < nfiles - 1 ? dc + npix : dc;
        orc_median27(ndet, nrows, dl, dc, dr, med);
        orc_resample(ndet, nrows, med, theta, shift, res);
        for (int jy = 0; jy < nrows; ++jy)
            memcpy(sino + ((size_t)jy * nfiles + job) * nx, res + (size_t)jy * nx, sizeof(float) * nx);
    }
    free(med); free(res);
}

/* ====================================================================== */
/* Cross-correlation registration (new; config 3's integer + parabolic      */
/* sub-pixel axis offset).  Not in the reference.                           */
/* ====================================================================== */

/* Products are truncated to 2^-32 fixed point and summed exactly in 128-bit
 * integers, so that the sums, and hence the integer argmax, do not depend on
 * summation order and cannot wrap.  A product that is not finite or not below
 * 2^31 in magnitude is out of range: the call returns 1 and leaves the
 * outputs unset (the library returns ACU_ERR_INVALID for the same inputs). */
typedef __int128 orc_i128;

/* The sum as a double: an exact int64 conversion when it fits int64, else
 * hi * 2^64 + lo (the library's conversion). */
static double i128_to_double(orc_i128 v)
{
    if (v >= (orc_i128)INT64_MIN && v <= (orc_i128)INT64_MAX) return (double)(int64_t)v;
    return ldexp((double)(int64_t)(v >> 64), 64) + (double)(uint64_t)v;
}

/* C(k) = sum_{x,y} p0(x,y) * p180(ndet-1-x+k, y), k = -kmax..kmax (0-based x);
 * terms with the mirrored index outside [0,ndet) are skipped.  Returns the
 * integer argmax (lowest k on ties) and the parabolic sub-pixel vertex.
 * The axis offset from the detector centre is (k + frac)/2 pixels.  corr
 * receives the sums as int64; returns 2 if one does not fit (the library's
 * ACU_ERR_UNSUPPORTED when corr_out is requested), 1 on out-of-range input. */
int orc_xcorr_register(int ndet, int nrows, const float *p0, const float *p180, int kmax,
                       int64_t *corr, int *k_best, double *k_sub)
{
    int nk = 2 * kmax + 1;
    orc_i128 *c = (orc_i128 *)malloc(sizeof(orc_i128) * (size_t)nk);
    int bad = 0;
    for (int i = 0; i < nk; ++i) {
        int k = i - kmax;
        orc_i128 acc = 0;
        for (int y = 0; y < nrows; ++y)
            for (int x = 0; x < ndet; ++x) {
                int xm = ndet - 1 - x + k;
                if (xm < 0 || xm >= ndet) continue;
                double p = (double)p0[(size_t)y * ndet + x] * (double)p180[(size_t)y * ndet + xm];
                if (fabs(p) < 2147483648.0) acc += (orc_i128)(int64_t)floor(p * 4294967296.0);
                else bad = 1;
            }
        c[i] = acc;
    }
    if (bad) {
        free(c);
        return 1;
    }
    int bi = 0;
    for (int i = 1; i < nk; ++i)
        if (c[i] > c[bi]) bi = i;
    int rc = 0;
    for (int i = 0; i < nk; ++i) {
        if (c[i] < (orc_i128)INT64_MIN || c[i] > (orc_i128)INT64_MAX) rc = 2;
        if (corr) corr[i] = (int64_t)c[i];
    }
    *k_best = bi - kmax;
    double frac = 0.0;
    if (bi > 0 && bi < nk - 1) {
        double cm = i128_to_double(c[bi - 1]), c0 = i128_to_double(c[bi]), cp = i128_to_double(c[bi + 1]);
        double den = cm - 2.0 * c0 + cp;
        if (den < 0.0) frac = 0.5 * (cm - cp) / den;
    }
    *k_sub = (double)(bi - kmax) + frac;
    free(c);
    return rc;
}

/* ====================================================================== */
/* Gradient of the registration-aware TV objective (FP64; new)             */
/* ====================================================================== */

/* Projector with per-angle detector offsets: bin jy of angle t is read at
 * detector coordinate jy + off[t].  off == 0 reproduces orc_radon_f64.    */
static void radon_off_f64(int N, int T, const float *theta, const double *u,
                          const double *off, double *sino)
{
    const double pi = 4.0 * atan(1.0);
    const double mid = (double)((N + 1) / 2);
#pragma omp parallel for schedule(static)
    for (int t = 0; t < T; ++t) {
        double ct = (pi * ((double)theta[t] - 90.0)) / 180.0;
        double c = cos(ct), s = sin(ct);
        for (int jy = 1; jy <= N; ++jy) {
            double sum = 0.0;
            double dy = ((double)jy + off[t]) - mid;
            for (int jx = 1; jx <= N; ++jx) {
                double xr = (c * ((double)jx - mid) - s * dy) + mid;
                double yr = (s * ((double)jx - mid) + c * dy) + mid;
                int y1 = (int)floor(yr), y2 = y1 + 1, x1 = (int)floor(xr), x2 = x1 + 1;
                int mn = x1 < y1 ? x1 : y1, mx = x2 > y2 ? x2 : y2;
                if (mn > 1 && mx < N + 1) {
                    double a = u[(size_t)(y1 - 1) * N + x1 - 1], b = u[(size_t)(y1 - 1) * N + x2 - 1];
                    double cc = u[(size_t)(y2 - 1) * N + x1 - 1], d = u[(size_t)(y2 - 1) * N + x2 - 1];
                    double wxl = x2 - xr, wxh = xr - x1, wyl = y2 - yr, wyh = yr - y1;
                    sum += a * wxl * wyl + b * wxh * wyl + cc * wxl * wyh + d * wxh * wyh;
                }
            }
            sino[(size_t)t * N + jy - 1] = sum / N;
        }
    }
}

/* loss = 1/2 ||A_off u - y||^2 + lambda * sum_i sqrt((Dx u)_i^2 + eps^2) + sqrt((Dy u)_i^2 + eps^2)
 * with the periodic backward differences of the reference's shrink step
 * (Dx u)(jx,jy) = u(jx-1,jy) - u(jx,jy).  Returns the loss; fills grad_u
 * (N*N) and grad_off (T) when non-NULL.                                    */
double orc_tv_loss_grad_f64(int N, int T, const float *theta, const double *u,
                            const double *off, const double *y, double lambda, double eps,
                            double *grad_u, double *grad_off)
{
    const double pi = 4.0 * atan(1.0);
    const double mid = (double)((N + 1) / 2);
    size_t NN = (size_t)N * N, NT = (size_t)N * T;
    double *res = (double *)malloc(sizeof(double) * NT);
    radon_off_f64(N, T, theta, u, off, res);
    double loss = 0.0;
    for (size_t i = 0; i < NT; ++i) { res[i] -= y[i]; loss += 0.5 * res[i] * res[i]; }
    if (grad_u) memset(grad_u, 0, sizeof(double) * NN);
    for (int t = 0; t < T; ++t) {
        double ct = (pi * ((double)theta[t] - 90.0)) / 180.0;
        double c = cos(ct), s = sin(ct);
        double go = 0.0;
        for (int jy = 1; jy <= N; ++jy) {
            double w = res[(size_t)t * N + jy - 1] / N;
            double dy = ((double)jy + off[t]) - mid;
            for (int jx = 1; jx <= N; ++jx) {
                double xr = (c * ((double)jx - mid) - s * dy) + mid;
                double yr = (s * ((double)jx - mid) + c * dy) + mid;
                int y1 = (int)floor(yr), y2 = y1 + 1, x1 = (int)floor(xr), x2 = x1 + 1;
                int mn = x1 < y1 ? x1 : y1, mx = x2 > y2 ? x2 : y2;
                if (mn > 1 && mx < N + 1) {
                    double wxl = x2 - xr, wxh = xr - x1, wyl = y2 - yr, wyh = yr - y1;
                    size_t i11 = (size_t)(y1 - 1) * N + x1 - 1, i21 = (size_t)(y1 - 1) * N + x2 - 1;
                    size_t i12 = (size_t)(y2 - 1) * N + x1 - 1, i22 = (size_t)(y2 - 1) * N + x2 - 1;
                    if (grad_u) {
                        grad_u[i11] += w * wxl * wyl; grad_u[i21] += w * wxh * wyl;
                        grad_u[i12] += w * wxl * wyh; grad_u[i22] += w * wxh * wyh;
                    }
                    if (grad_off) {
                        double gx = (u[i21] - u[i11]) * wyl + (u[i22] - u[i12]) * wyh;
                        double gy = (u[i12] - u[i11]) * wxl + (u[i22] - u[i21]) * wxh;
                        /* d(xr)/d(off) = -s, d(yr)/d(off) = c */
                        go += w * (gx * (-s) + gy * c);
                    }
                }
            }
        }
        if (grad_off) grad_off[t] = go;
    }
    free(res);
    for (int jy = 1; jy <= N; ++jy)
        for (int jx = 1; jx <= N; ++jx) {
            int jxl = jx - 1 + N - ((jx - 1 + N) / (N + 1)) * N;
            int jyl = jy - 1 + N - ((jy - 1 + N) / (N + 1)) * N;
            size_t i = (size_t)(jy - 1) * N + jx - 1;
            size_t ixl = (size_t)(jy - 1) * N + jxl - 1, iyl = (size_t)(jyl - 1) * N + jx - 1;
            double gx = u[ixl] - u[i], gy = u[iyl] - u[i];
            double nx = sqrt(gx * gx + eps * eps), ny = sqrt(gy * gy + eps * eps);
            loss += lambda * (nx + ny);
            if (grad_u) {
                grad_u[ixl] += lambda * gx / nx; grad_u[i] -= lambda * gx / nx;
                grad_u[iyl] += lambda * gy / ny; grad_u[i] -= lambda * gy / ny;
            }
        }
    return loss;
}

int orc_version(void) { return 1; }
