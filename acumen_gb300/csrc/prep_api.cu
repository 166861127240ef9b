// C ABI of the projection-preprocessing path: tomography/fits_to_hpc.F90
// (flat/dark averages, log-normalisation) and
// tomography/projections_to_sinogram_hpc.F90 (0/180-degree projections,
// rotation-axis registration, 27-point median, resample, transpose).
#include <cmath>
#include <cstring>

#include "ctx.h"
#include "prep.h"

using namespace acu;

namespace {

int check_any(acu_ctx* c)
{
    if (!c) return set_err(nullptr, ACU_ERR_INVALID, "null context");
    return ACU_OK;
}

int check_proj(acu_ctx* c, int ndet, int nrows)
{
    CKRET(check_any(c));
    if (ndet < 2 || nrows < 1) return set_err(c, ACU_ERR_INVALID, "invalid projection size %d x %d", ndet, nrows);
    return ACU_OK;
}

// tomography/tv_hpc.F90:546-547: first index (1-based) minimising |theta - target|
int minloc_abs(int n, const float* theta, float target)
{
    int best = 1;
    float bv = std::fabs(theta[0] - target);
    for (int j = 2; j <= n; ++j) {
        const float v = std::fabs(theta[j - 1] - target);
        if (v < bv) {
            bv = v;
            best = j;
        }
    }
    return best;
}

double read_scalar(acu_ctx* c, const double* d, int* rc)
{
    double h = 0.0;
    cudaError_t e = cudaMemcpyAsync(&h, d, sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    *rc = e == cudaSuccess ? ACU_OK : set_err(c, ACU_ERR_CUDA, "scalar read failed: %s", cudaGetErrorString(e));
    return h;
}

// Objective of the pattern search for one candidate, as the reference's
// single-precision `error_diff` (accumulated in FP64, rounded once).
int mirror_error(acu_ctx* c, int ndet, int nrows, const float* p0, const float* p180, float th, float shift,
                 float* out)
{
    const int nblk = mirror_error_blocks(ndet, nrows);
    CK(c, c->w_part.ensure(sizeof(double) * (nblk + 8)));
    double* part = c->w_part.as<double>();
    launch_mirror_error(ndet, nrows, p0, p180, std::cos(th), std::sin(th), shift, part, nblk, part + nblk,
                        c->stream);
    CKLAUNCH(c);
    int rc;
    const double e = read_scalar(c, part + nblk, &rc);
    if (rc != ACU_OK) return rc;
    *out = (float)e;
    return ACU_OK;
}

}  // namespace

extern "C" {

int acu_frame_average_u16_dev(acu_ctx* c, int nframes, long npix, const uint16_t* d_frames, float* d_out)
{
    CKRET(check_any(c));
    if (nframes < 1 || npix < 0 || !d_frames || !d_out) return set_err(c, ACU_ERR_INVALID, "invalid frame stack");
    launch_frame_average_u16(nframes, npix, d_frames, d_out, c->stream);
    CKLAUNCH(c);
    return ACU_OK;
}

int acu_frame_average_dev(acu_ctx* c, int nframes, long npix, const float* d_frames, float* d_out)
{
    CKRET(check_any(c));
    if (nframes < 1 || npix < 0 || !d_frames || !d_out) return set_err(c, ACU_ERR_INVALID, "invalid frame stack");
    launch_frame_average_f32(nframes, npix, d_frames, d_out, c->stream);
    CKLAUNCH(c);
    return ACU_OK;
}

int acu_normalize_u16_dev(acu_ctx* c, int mode, int nproj, long npix, const uint16_t* d_raw, const float* d_ob,
                          const float* d_df, float* d_out)
{
    CKRET(check_any(c));
    if ((mode != 0 && mode != 1) || nproj < 0 || npix < 0 || !d_raw || !d_ob || !d_out || (mode == 1 && !d_df))
        return set_err(c, ACU_ERR_INVALID, "invalid normalisation arguments (mode %d)", mode);
    launch_normalize_u16(mode, nproj, npix, d_raw, d_ob, d_df, d_out, c->stream);
    CKLAUNCH(c);
    return ACU_OK;
}

int acu_normalize_dev(acu_ctx* c, int mode, int nproj, long npix, const float* d_raw, const float* d_ob,
                      const float* d_df, float* d_out)
{
    CKRET(check_any(c));
    if ((mode != 0 && mode != 1) || nproj < 0 || npix < 0 || !d_raw || !d_ob || !d_out || (mode == 1 && !d_df))
        return set_err(c, ACU_ERR_INVALID, "invalid normalisation arguments (mode %d)", mode);
    launch_normalize_f32(mode, nproj, npix, d_raw, d_ob, d_df, d_out, c->stream);
    CKLAUNCH(c);
    return ACU_OK;
}

int acu_pick_angle_dev(acu_ctx* c, int nfiles, const float* theta, long npix, const float* d_proj, float target,
                       float* d_out)
{
    CKRET(check_any(c));
    if (nfiles < 1 || !theta || !d_proj || !d_out || npix < 0)
        return set_err(c, ACU_ERR_INVALID, "invalid projection stack");
    const int js = minloc_abs(nfiles, theta, target);
    int ia = -1, ib = -1;
    if (theta[js - 1] != target) {
        if (theta[js - 1] <= target) {
            if (js < nfiles) { ia = js - 1; ib = js; }
        } else if (js > 1) {
            ia = js - 2; ib = js - 1;
        }
    }
    if (ia < 0) {
        CK(c, cudaMemcpyAsync(d_out, d_proj + (size_t)(js - 1) * npix, sizeof(float) * npix,
                              cudaMemcpyDeviceToDevice, c->stream));
        return ACU_OK;
    }
    launch_lerp(npix, d_proj + (size_t)ia * npix, d_proj + (size_t)ib * npix, theta[ia], theta[ib], target, d_out,
                c->stream);
    CKLAUNCH(c);
    return ACU_OK;
}

int acu_resample_dev(acu_ctx* c, int ndet, int nrows, const float* d_src, float theta, float shift, float* d_out)
{
    CKRET(check_proj(c, ndet, nrows));
    if (!d_src || !d_out) return set_err(c, ACU_ERR_INVALID, "null array");
    launch_resample(ndet, nrows, d_src, std::cos(theta), std::sin(theta), shift, d_out, c->stream);
    CKLAUNCH(c);
    return ACU_OK;
}

int acu_register_dev(acu_ctx* c, int ndet, int nrows, const float* d_p0, const float* d_p180, float* theta_out,
                     float* shift_out, int* evals_out)
{
    CKRET(check_proj(c, ndet, nrows));
    if (!d_p0 || !d_p180 || !theta_out || !shift_out) return set_err(c, ACU_ERR_INVALID, "null argument");
    const int add = (ndet % 2 == 0) ? 1 : 0;
    // centre of mass (:231-248)
    const int nblk = mirror_error_blocks(ndet, nrows);
    CK(c, c->w_part.ensure(sizeof(double) * (3 * nblk + 8)));
    double* part = c->w_part.as<double>();
    launch_com(ndet, nrows, d_p0, d_p180, part, nblk, part + 3 * nblk, c->stream);
    CKLAUNCH(c);
    double sums[3];
    CK(c, cudaMemcpyAsync(sums, part + 3 * nblk, sizeof sums, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    (void)add;
    const float tm = (float)sums[0], cmx0 = (float)sums[1], cmx180 = (float)sums[2];
    const float shift_scale = (float)ndet;
    float best_shift = -((cmx0 / tm + cmx180 / tm) / (2.0f * shift_scale));
    float best_theta = 0.0f;
    float dshift = 1e-4f, dtheta = 1e-4f;
    const int n_sp = 6;
    const float n_mag = 1.05f, n_min = 2.0f / (float)n_sp;
    int ne = 1;
    float best_error;
    CKRET(mirror_error(c, ndet, nrows, d_p0, d_p180, best_theta, best_shift, &best_error));
    // multiplicative pattern search (:287-364)
    while (std::fmax(dtheta, dshift) > 1e-8f) {
        float perr = best_error;
        for (int jsp = 1; jsp <= n_sp; ++jsp) {
            const float th = best_theta + dtheta * (float)(jsp - n_sp / 2);
            float e;
            CKRET(mirror_error(c, ndet, nrows, d_p0, d_p180, th, best_shift, &e));
            ++ne;
            if (e < best_error) {
                best_theta = th;
                best_error = e;
            }
        }
        dtheta = (best_error < perr) ? n_mag * dtheta : n_min * dtheta;
        perr = best_error;
        for (int jsp = 1; jsp <= n_sp; ++jsp) {
            const float sh = best_shift + dshift * (float)(jsp - n_sp / 2);
            float e;
            CKRET(mirror_error(c, ndet, nrows, d_p0, d_p180, best_theta, sh, &e));
            ++ne;
            if (e < best_error) {
                best_shift = sh;
                best_error = e;
            }
        }
        dshift = (best_error < perr) ? n_mag * dshift : n_min * dshift;
        if (ne > 200000) return set_err(c, ACU_ERR_TIMEOUT, "registration did not converge in 200000 evaluations");
    }
    *theta_out = best_theta;
    *shift_out = best_shift;
    if (evals_out) *evals_out = ne;
    return ACU_OK;
}

int acu_xcorr_register_dev(acu_ctx* c, int ndet, int nrows, const float* d_p0, const float* d_p180, int kmax,
                           int64_t* corr_out, int* k_best, double* k_sub)
{
    CKRET(check_proj(c, ndet, nrows));
    if (!d_p0 || !d_p180 || !k_best || !k_sub || kmax < 1 || kmax > 4096)
        return set_err(c, ACU_ERR_INVALID, "invalid cross-correlation arguments (kmax %d)", kmax);
    const size_t nw = xcorr_scratch_words(kmax);
    CK(c, c->w_part.ensure(sizeof(unsigned long long) * nw));
    unsigned long long* w = c->w_part.as<unsigned long long>();
    CK(c, launch_xcorr(ndet, nrows, kmax, d_p0, d_p180, w, c->stream));
    std::vector<unsigned long long> h(nw);
    CK(c, cudaMemcpyAsync(h.data(), w, sizeof(unsigned long long) * nw, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    const char* why = "";
    const int rc = xcorr_finish(kmax, h.data(), corr_out, k_best, k_sub, &why);
    if (rc != ACU_OK) return set_err(c, rc, "cross-correlation registration: %s", why);
    return ACU_OK;
}

int acu_median27_dev(acu_ctx* c, int ndet, int nrows, const float* d_l, const float* d_c, const float* d_r,
                     float* d_out)
{
    CKRET(check_proj(c, ndet, nrows));
    if (!d_l || !d_c || !d_r || !d_out) return set_err(c, ACU_ERR_INVALID, "null array");
    // the kernel walks a projection stack; present the three images as a
    // three-projection stack when they are consecutive, else copy them
    const size_t npix = (size_t)ndet * nrows;
    if (d_l + npix == d_c && d_c + npix == d_r) {
        launch_median27(ndet, nrows, 1, 1, 3, d_l, d_out, c->stream);
    } else {
        CK(c, c->w_in.ensure(sizeof(float) * 3 * npix));
        float* st = c->w_in.as<float>();
        CK(c, cudaMemcpyAsync(st, d_l, sizeof(float) * npix, cudaMemcpyDeviceToDevice, c->stream));
        CK(c, cudaMemcpyAsync(st + npix, d_c, sizeof(float) * npix, cudaMemcpyDeviceToDevice, c->stream));
        CK(c, cudaMemcpyAsync(st + 2 * npix, d_r, sizeof(float) * npix, cudaMemcpyDeviceToDevice, c->stream));
        launch_median27(ndet, nrows, 1, 1, 3, st, d_out, c->stream);
    }
    CKLAUNCH(c);
    return ACU_OK;
}

int acu_proj_to_sino_dev(acu_ctx* c, int nproj, int ndet, int nrows, const float* d_proj, float theta, float shift,
                         float* d_sino)
{
    CKRET(check_proj(c, ndet, nrows));
    if (nproj < 1 || !d_proj || !d_sino) return set_err(c, ACU_ERR_INVALID, "invalid projection stack");
    const size_t npix = (size_t)ndet * nrows;
    const int chunk = (int)std::max<size_t>(1, std::min<size_t>(nproj, (size_t)(512u << 20) / (npix * 4)));
    CK(c, c->w_q.ensure(sizeof(float) * npix * chunk));
    float* med = c->w_q.as<float>();
    const float cth = std::cos(theta), sth = std::sin(theta);
    for (int p0 = 0; p0 < nproj; p0 += chunk) {
        const int n = std::min(chunk, nproj - p0);
        launch_median27(ndet, nrows, n, p0, nproj, d_proj, med, c->stream);
        launch_resample_to_sino(ndet, nrows, n, p0, nproj, med, cth, sth, shift, d_sino, c->stream);
        CKLAUNCH(c);
    }
    return ACU_OK;
}

int acu_normalize_stack_u16(acu_ctx* c, int mode, int nproj, long npix, const uint16_t* raw, int nflat,
                            const uint16_t* flats, int ndark, const uint16_t* darks, float* out)
{
    CKRET(check_any(c));
    if ((mode != 0 && mode != 1) || nproj < 0 || npix < 1 || !raw || nflat < 1 || !flats || !out ||
        (mode == 1 && (ndark < 1 || !darks)))
        return set_err(c, ACU_ERR_INVALID, "invalid normalisation arguments (mode %d)", mode);
    if (nproj == 0) return ACU_OK;
    DevBuf d_raw, d_fl, d_dk, d_ob, d_df, d_out;
    cudaStream_t st = c->stream;
    CK(c, d_fl.ensure(sizeof(uint16_t) * npix * nflat));
    CK(c, d_ob.ensure(sizeof(float) * npix));
    CK(c, d_df.ensure(sizeof(float) * npix));
    CK(c, cudaMemcpyAsync(d_fl.p, flats, sizeof(uint16_t) * npix * nflat, cudaMemcpyHostToDevice, st));
    launch_frame_average_u16(nflat, npix, d_fl.as<uint16_t>(), d_ob.as<float>(), st);
    if (ndark > 0 && darks) {
        CK(c, d_dk.ensure(sizeof(uint16_t) * npix * ndark));
        CK(c, cudaMemcpyAsync(d_dk.p, darks, sizeof(uint16_t) * npix * ndark, cudaMemcpyHostToDevice, st));
        launch_frame_average_u16(ndark, npix, d_dk.as<uint16_t>(), d_df.as<float>(), st);
    } else {
        CK(c, cudaMemsetAsync(d_df.p, 0, sizeof(float) * npix, st));
    }
    // stream the projections through in chunks of <= 1 GiB of output
    const long chunk = std::max<long>(1, (long)((1u << 30) / (npix * sizeof(float))));
    const long nc = std::min<long>(chunk, nproj);
    CK(c, d_raw.ensure(sizeof(uint16_t) * npix * nc));
    CK(c, d_out.ensure(sizeof(float) * npix * nc));
    for (long p0 = 0; p0 < nproj; p0 += nc) {
        const long n = std::min<long>(nc, nproj - p0);
        CK(c, cudaMemcpyAsync(d_raw.p, raw + (size_t)p0 * npix, sizeof(uint16_t) * npix * n, cudaMemcpyHostToDevice,
                              st));
        launch_normalize_u16(mode, (int)n, npix, d_raw.as<uint16_t>(), d_ob.as<float>(), d_df.as<float>(),
                             d_out.as<float>(), st);
        CKLAUNCH(c);
        CK(c, cudaMemcpyAsync(out + (size_t)p0 * npix, d_out.p, sizeof(float) * npix * n, cudaMemcpyDeviceToHost, st));
    }
    CK(c, cudaStreamSynchronize(st));
    return ACU_OK;
}

int acu_normalize_stack(acu_ctx* c, int mode, int nproj, long npix, const float* raw, const float* ob,
                        const float* df, float* out)
{
    CKRET(check_any(c));
    if ((mode != 0 && mode != 1) || nproj < 0 || npix < 1 || !raw || !ob || !out || (mode == 1 && !df))
        return set_err(c, ACU_ERR_INVALID, "invalid normalisation arguments (mode %d)", mode);
    if (nproj == 0) return ACU_OK;
    DevBuf d_raw, d_ob, d_df, d_out;
    cudaStream_t st = c->stream;
    CK(c, d_ob.ensure(sizeof(float) * npix));
    CK(c, d_df.ensure(sizeof(float) * npix));
    CK(c, cudaMemcpyAsync(d_ob.p, ob, sizeof(float) * npix, cudaMemcpyHostToDevice, st));
    if (df)
        CK(c, cudaMemcpyAsync(d_df.p, df, sizeof(float) * npix, cudaMemcpyHostToDevice, st));
    else
        CK(c, cudaMemsetAsync(d_df.p, 0, sizeof(float) * npix, st));
    const long chunk = std::max<long>(1, (long)((1u << 30) / (npix * sizeof(float))));
    const long nc = std::min<long>(chunk, nproj);
    CK(c, d_raw.ensure(sizeof(float) * npix * nc));
    CK(c, d_out.ensure(sizeof(float) * npix * nc));
    for (long p0 = 0; p0 < nproj; p0 += nc) {
        const long n = std::min<long>(nc, nproj - p0);
        CK(c, cudaMemcpyAsync(d_raw.p, raw + (size_t)p0 * npix, sizeof(float) * npix * n, cudaMemcpyHostToDevice, st));
        launch_normalize_f32(mode, (int)n, npix, d_raw.as<float>(), d_ob.as<float>(), d_df.as<float>(),
                             d_out.as<float>(), st);
        CKLAUNCH(c);
        CK(c, cudaMemcpyAsync(out + (size_t)p0 * npix, d_out.p, sizeof(float) * npix * n, cudaMemcpyDeviceToHost, st));
    }
    CK(c, cudaStreamSynchronize(st));
    return ACU_OK;
}

int acu_proj_to_sino(acu_ctx* c, int nproj, int ndet, int nrows, const float* proj, const float* theta_deg,
                     int reg_method, float* sino_out, float* theta_out, float* shift_out)
{
    CKRET(check_proj(c, ndet, nrows));
    if (nproj < 1 || !proj || !theta_deg || !sino_out) return set_err(c, ACU_ERR_INVALID, "invalid arguments");
    if (reg_method != 0 && reg_method != 1) return set_err(c, ACU_ERR_INVALID, "reg_method must be 0 or 1");
    const size_t npix = (size_t)ndet * nrows;
    const int add = ndet % 2 == 0 ? 1 : 0;
    const size_t nsino = (size_t)nrows * nproj * (ndet + add);
    DevBuf d_proj, d_p0, d_p180, d_sino;
    CK(c, d_proj.ensure(sizeof(float) * npix * nproj));
    CK(c, d_p0.ensure(sizeof(float) * npix));
    CK(c, d_p180.ensure(sizeof(float) * npix));
    CK(c, d_sino.ensure(sizeof(float) * nsino));
    cudaStream_t st = c->stream;
    CK(c, cudaMemcpyAsync(d_proj.p, proj, sizeof(float) * npix * nproj, cudaMemcpyHostToDevice, st));
    CKRET(acu_pick_angle_dev(c, nproj, theta_deg, (long)npix, d_proj.as<float>(), 0.0f, d_p0.as<float>()));
    CKRET(acu_pick_angle_dev(c, nproj, theta_deg, (long)npix, d_proj.as<float>(), 180.0f, d_p180.as<float>()));
    float th = 0.0f, sh = 0.0f;
    if (reg_method == 0) {
        CKRET(acu_register_dev(c, ndet, nrows, d_p0.as<float>(), d_p180.as<float>(), &th, &sh, nullptr));
    } else {
        int kb;
        double ks;
        const int kmax = std::max(1, std::min(ndet / 4, 512));
        CKRET(acu_xcorr_register_dev(c, ndet, nrows, d_p0.as<float>(), d_p180.as<float>(), kmax, nullptr, &kb, &ks));
        sh = (float)(((double)add - ks) / (2.0 * ndet));
    }
    CKRET(acu_proj_to_sino_dev(c, nproj, ndet, nrows, d_proj.as<float>(), th, sh, d_sino.as<float>()));
    CK(c, cudaMemcpyAsync(sino_out, d_sino.p, sizeof(float) * nsino, cudaMemcpyDeviceToHost, st));
    CK(c, cudaStreamSynchronize(st));
    if (theta_out) *theta_out = th;
    if (shift_out) *shift_out = sh;
    return ACU_OK;
}

int acu_proj_to_sino_u16(acu_ctx* c, int nproj, int ndet, int nrows, const uint16_t* raw, const float* theta_deg,
                         int nflat, const uint16_t* flats, int ndark, const uint16_t* darks, int norm_mode,
                         int reg_method, float* sino_out, float* theta_out, float* shift_out)
{
    CKRET(check_proj(c, ndet, nrows));
    if (nproj < 1 || !raw || !theta_deg || nflat < 1 || !flats || !sino_out || (norm_mode == 1 && (ndark < 1 || !darks)))
        return set_err(c, ACU_ERR_INVALID, "invalid pipeline arguments");
    if (reg_method != 0 && reg_method != 1) return set_err(c, ACU_ERR_INVALID, "reg_method must be 0 or 1");
    const size_t npix = (size_t)ndet * nrows;
    const int add = ndet % 2 == 0 ? 1 : 0;
    const size_t nsino = (size_t)nrows * nproj * (ndet + add);
    DevBuf d_raw, d_fl, d_dk, d_ob, d_df, d_proj, d_p0, d_p180, d_sino;
    CK(c, d_raw.ensure(sizeof(uint16_t) * npix * nproj));
    CK(c, d_fl.ensure(sizeof(uint16_t) * npix * nflat));
    CK(c, d_ob.ensure(sizeof(float) * npix));
    CK(c, d_df.ensure(sizeof(float) * npix));
    CK(c, d_proj.ensure(sizeof(float) * npix * nproj));
    CK(c, d_p0.ensure(sizeof(float) * npix));
    CK(c, d_p180.ensure(sizeof(float) * npix));
    CK(c, d_sino.ensure(sizeof(float) * nsino));
    cudaStream_t st = c->stream;
    CK(c, cudaMemcpyAsync(d_raw.p, raw, sizeof(uint16_t) * npix * nproj, cudaMemcpyHostToDevice, st));
    CK(c, cudaMemcpyAsync(d_fl.p, flats, sizeof(uint16_t) * npix * nflat, cudaMemcpyHostToDevice, st));
    launch_frame_average_u16(nflat, (long)npix, d_fl.as<uint16_t>(), d_ob.as<float>(), st);
    if (ndark > 0 && darks) {
        CK(c, d_dk.ensure(sizeof(uint16_t) * npix * ndark));
        CK(c, cudaMemcpyAsync(d_dk.p, darks, sizeof(uint16_t) * npix * ndark, cudaMemcpyHostToDevice, st));
        launch_frame_average_u16(ndark, (long)npix, d_dk.as<uint16_t>(), d_df.as<float>(), st);
    } else {
        CK(c, cudaMemsetAsync(d_df.p, 0, sizeof(float) * npix, st));
    }
    launch_normalize_u16(norm_mode, nproj, (long)npix, d_raw.as<uint16_t>(), d_ob.as<float>(), d_df.as<float>(),
                         d_proj.as<float>(), st);
    CKLAUNCH(c);
    CKRET(acu_pick_angle_dev(c, nproj, theta_deg, (long)npix, d_proj.as<float>(), 0.0f, d_p0.as<float>()));
    CKRET(acu_pick_angle_dev(c, nproj, theta_deg, (long)npix, d_proj.as<float>(), 180.0f, d_p180.as<float>()));
    float th = 0.0f, sh = 0.0f;
    if (reg_method == 0) {
        CKRET(acu_register_dev(c, ndet, nrows, d_p0.as<float>(), d_p180.as<float>(), &th, &sh, nullptr));
    } else {
        int kb;
        double ks;
        const int kmax = std::max(1, std::min(ndet / 4, 512));
        CKRET(acu_xcorr_register_dev(c, ndet, nrows, d_p0.as<float>(), d_p180.as<float>(), kmax, nullptr, &kb, &ks));
        sh = (float)(((double)add - ks) / (2.0 * ndet));
    }
    CKRET(acu_proj_to_sino_dev(c, nproj, ndet, nrows, d_proj.as<float>(), th, sh, d_sino.as<float>()));
    CK(c, cudaMemcpyAsync(sino_out, d_sino.p, sizeof(float) * nsino, cudaMemcpyDeviceToHost, st));
    CK(c, cudaStreamSynchronize(st));
    if (theta_out) *theta_out = th;
    if (shift_out) *shift_out = sh;
    return ACU_OK;
}

}  // extern "C"
