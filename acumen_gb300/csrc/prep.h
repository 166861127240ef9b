// Launchers of the projection-preprocessing kernels (kernels_prep.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace acu {

void launch_frame_average_u16(int nf, long npix, const uint16_t* f, float* out, cudaStream_t st);
void launch_frame_average_f32(int nf, long npix, const float* f, float* out, cudaStream_t st);
void launch_normalize_u16(int mode, int nproj, long npix, const uint16_t* raw, const float* ob, const float* df,
                          float* out, cudaStream_t st);
void launch_normalize_f32(int mode, int nproj, long npix, const float* raw, const float* ob, const float* df,
                          float* out, cudaStream_t st);
void launch_lerp(long n, const float* a, const float* b, float ta, float tb, float target, float* out,
                 cudaStream_t st);
void launch_resample(int ndet, int nrows, const float* src, float cth, float sth, float shift, float* out,
                     cudaStream_t st);
int mirror_error_blocks(int ndet, int nrows);
// writes the FP64 mismatch to out[0]; part holds nblk partials (scratch)
void launch_mirror_error(int ndet, int nrows, const float* p0, const float* p180, float cth, float sth, float shift,
                         double* part, int nblk, double* out, cudaStream_t st);
// writes tm, cmx_0, cmx_180 to out3[0..2]; part holds 3 * nblk partials
void launch_com(int ndet, int nrows, const float* p0, const float* p180, double* part, int nblk, double* out3,
                cudaStream_t st);
// Cross-correlation registration: scratch holds xcorr_scratch_words(kmax)
// 64-bit words (per-lag 128-bit sums, argmax index and range flag); the
// launcher clears it first and returns the first failing call's error.
// xcorr_finish turns a host copy of the scratch into the results (ACU_OK, or
// an ACU_ERR_* code with the reason in *why).
size_t xcorr_scratch_words(int kmax);
cudaError_t launch_xcorr(int ndet, int nrows, int kmax, const float* p0, const float* p180,
                         unsigned long long* scratch, cudaStream_t st);
int xcorr_finish(int kmax, const unsigned long long* scratch, int64_t* corr_out, int* k_best, double* k_sub,
                 const char** why);
void launch_median27(int ndet, int nrows, int nchunk, int p_first, int nfiles, const float* proj, float* out,
                     cudaStream_t st);
void launch_resample_to_sino(int ndet, int nrows, int nchunk, int p_first, int nfiles, const float* med,
                             float cth, float sth, float shift, float* sino, cudaStream_t st);

}  // namespace acu
