/*
 * acumen_gpu.h -- C ABI of the GB300 tomography library (libacumen_gpu.so).
 *
 * Drop-in replacement for the compute of the reference's Fortran module
 * `Tomography` (tomography/tv_hpc.F90:1-390) and of the inline kernels of
 * tomography/projections_to_sinogram_hpc.F90 and tomography/fits_to_hpc.F90.
 * The reference exposes no C interface: its callers are the Fortran driver
 * programs, which bind these entry points through ISO_C_BINDING (the
 * interface module is acumen_gb300/fortran/acumen_gpu.f90).
 *
 * Conventions
 *  - Every function returns int: ACU_OK (0) or a negative ACU_ERR_* code;
 *    acu_last_error(ctx) gives the message (acu_last_error(NULL) for errors
 *    raised before a context exists).  Nothing aborts the process.
 *  - Arrays are single precision in the reference's Fortran order, first index
 *    fastest: image img(jx,jy) is N*N floats with x fastest; sinogram
 *    sino(jbin,jtheta) is T*N floats with the bin fastest; S slices are
 *    stored one after another.  Angles are degrees, as in theta.dat.
 *  - Functions without a suffix take HOST pointers: they copy in, compute and
 *    copy out, and return when the results are in host memory.  The `_dev`
 *    variants take DEVICE pointers, are ordered on the context's stream and
 *    do not synchronise.  `_f64` variants run the same kernels in double
 *    precision on double arrays (used to check the single-precision path).
 *  - A context is used by one host thread at a time; contexts are
 *    independent.  The library owns its device work buffers.
 */
#ifndef ACUMEN_GPU_H
#define ACUMEN_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ACU_OK 0
#define ACU_ERR_INVALID (-1)     /* bad argument (size, pointer, mode) */
#define ACU_ERR_CUDA (-2)        /* a CUDA runtime call failed */
#define ACU_ERR_NOMEM (-3)       /* device or host allocation failed */
#define ACU_ERR_TIMEOUT (-4)     /* a bounded device wait gave up */
#define ACU_ERR_UNSUPPORTED (-5) /* valid request this build does not handle */

typedef struct acu_ctx acu_ctx;

/* ---- context: tomography/tv_hpc.F90:11-82 (int_radon / fin_radon) ---------
 * Creates the geometry of one reconstruction grid: nimage = N (the grid side,
 * equal to the number of detector bins), ntheta = T angles theta_deg[T],
 * taper width wpu of the circular mask.  Computes the filter taps and mask
 * (int_radon, tv_hpc.F90:53-74).  nimage = 0 creates a context without a
 * grid, for the preprocessing functions only.                               */
int acu_ctx_create(acu_ctx **ctx, int nimage, int ntheta, const float *theta_deg, int wpu);
/* tv_hpc.F90:80-82 (fin_radon): releases every device buffer of ctx. */
int acu_ctx_destroy(acu_ctx *ctx);
const char *acu_last_error(const acu_ctx *ctx);
/* Orders all later work of ctx on this cudaStream_t; NULL (the default) is the
 * legacy default stream.  CUDA graphs are captured on a private stream and
 * launched on this one. */
int acu_set_stream(acu_ctx *ctx, void *cuda_stream);

#define ACU_OPT_FILTER 1    /* 0: FFT ramp filter (default); 1: direct O(N^2) sum (tv_hpc.F90:93-105) */
#define ACU_OPT_LANES 2     /* slices per thread in batched kernels: 0 auto (default), 1 or 4 */
#define ACU_OPT_GRAPH 3     /* 1: capture the Bregman outer iteration as a CUDA graph (default); 0: launch */
#define ACU_OPT_VERBOSE 4   /* 1: print the reference's "Slice/Loop/delta" lines (tv_hpc.F90:350-352) */
#define ACU_OPT_PRINT_EVERY 5 /* outer-loop period of those lines: 50 (tv_hpc) or 10 (tv_hpc_slice) */
#define ACU_OPT_SLICE_BASE 6  /* slice number printed for the first slice of a call (default 1) */
#define ACU_OPT_PROJECTOR 7   /* single-precision batched projector: 0 pair images, 1 image + transpose,
                                 2 the same with the taps loaded by row parity, 3 the same with the taps
                                 of the previous sample reused, 4 reuse with each warp's steps limited
                                 to those that can meet a valid cell, 5 the same with paired FP32 FMAs
                                 (fma.rn.f32x2), 6 pixel lines of 32 slices walked in bands of rows,
                                 7 automatic (default): 6 when the batch fills its 32-slice lines to
                                 8/9 or more, else 5; 1 and 3 to 6 give identical results */
#define ACU_OPT_POSITIONS 8   /* single-precision sample positions: 1 exact (default; coordinates from split
                                 FP64 angle tables, within ~1e-7 px of FP64, and the FFT filter's spectrum
                                 from FP64-evaluated taps: the mode that meets relL2 1e-5 FBP / 1e-4 TV
                                 against FP64 at the benchmark sizes), 0 the reference's single-precision
                                 arithmetic (tv_hpc.F90:53-56,113-115,144-146), whose rounding of the
                                 coordinate at magnitude ~N moves samples by ~6e-5 px */
#define ACU_OPT_RESIDUAL 9    /* batched TV: the initial CG residual mu*iradon(fk) - mu*iradon(radon(uk)) as
                                 2 iradon(f - radon(uk)) + iradon(fk - f), both carried through the CG and
                                 Bregman updates and recomputed with radon(uk) every ACU_OPT_RADON_REFRESH
                                 outer iterations (default; as 1 when radon(uk) is not carried),
                                 1 one backprojection of fk - radon(uk), or 0 the reference's two */
#define ACU_OPT_BP_GROUPS 10  /* 4-slice groups per backprojection thread: 0 auto (default: 1 with the
                                 angle table in the launch parameters, else 2 where the groups divide),
                                 1, 2 or 4; the groups share the angle's table entry and sample
                                 position, the sums are unchanged */
#define ACU_OPT_RADON_REFRESH 11 /* batched TV: radon(uk) for the Bregman update recomputed every outer
                                 iteration (1, the reference), or carried through the CG updates
                                 (radon(uk + a p) = radon(uk) + a radon(p)) and recomputed every K-th
                                 outer iteration (K >= 2, default 5; 0 never) */
#define ACU_OPT_BP_PARAM_TABLE 12 /* single-precision backprojection: 1 passes the per-angle table in the launch's
                                 parameters when T <= 1920 (constant-cache reads, default), 0 reads
                                 it from device memory; the results are identical */
#define ACU_OPT_MAX_BATCH 13  /* acu_tvopt / acu_tvopt_dev / acu_tvopt_plain: at most this many slices on
                                 the device at a time (0, default: as many as fit in the free device
                                 memory); larger calls are solved in consecutive chunks of slices, each
                                 slice as in one batch */
#define ACU_OPT_BP_STAGED 14  /* exact single-precision backprojection with the angle table in the launch
                                 parameters: 1 stages each angle's sinogram bins of a 32x8 pixel tile in
                                 shared memory with bulk copies (cp.async.bulk, double-buffered, mbarrier
                                 waits bounded), 0 reads them through L1 (default); identical results */
int acu_set_option(acu_ctx *ctx, int option, int value);
int acu_get_option(const acu_ctx *ctx, int option, int *value);

/* ---- Radon operators -------------------------------------------------------
 * acu_iradon: tomography/tv_hpc.F90:84-126 (iradon) -- ramp filter along each
 *   sinogram column, pixel-driven linear-interpolation backprojection, times
 *   the tapered mask.  sino: S*T*N, img: S*N*N.  Also get_slice
 *   (tv_hpc.F90:365-386, fbp_hpc.F90:129-150), which is iradon with copies.
 * acu_radon: tomography/tv_hpc.F90:129-159 (radon) -- bilinear ray sums / N.
 * acu_radon_adjoint: exact transpose of acu_radon (new; not in the reference):
 *   <radon(x), y> = <x, radon_adjoint(y)> up to round-off.
 * acu_filter_dev / acu_backproject_dev: the two halves of iradon
 *   (tv_hpc.F90:93-105 and :107-123).                                         */
int acu_iradon(acu_ctx *ctx, int nslices, const float *sino, float *img);
int acu_radon(acu_ctx *ctx, int nslices, const float *img, float *sino);
int acu_radon_adjoint(acu_ctx *ctx, int nslices, const float *sino, float *img);
int acu_iradon_dev(acu_ctx *ctx, int nslices, const float *d_sino, float *d_img);
int acu_radon_dev(acu_ctx *ctx, int nslices, const float *d_img, float *d_sino);
int acu_radon_adjoint_dev(acu_ctx *ctx, int nslices, const float *d_sino, float *d_img);
int acu_filter_dev(acu_ctx *ctx, int nslices, const float *d_sino, float *d_out);
int acu_backproject_dev(acu_ctx *ctx, int nslices, const float *d_filtered, float *d_img);
int acu_iradon_dev_f64(acu_ctx *ctx, int nslices, const double *d_sino, double *d_img);
int acu_radon_dev_f64(acu_ctx *ctx, int nslices, const double *d_img, double *d_sino);
int acu_radon_adjoint_dev_f64(acu_ctx *ctx, int nslices, const double *d_sino, double *d_img);
int acu_filter_dev_f64(acu_ctx *ctx, int nslices, const double *d_sino, double *d_out);
int acu_backproject_dev_f64(acu_ctx *ctx, int nslices, const double *d_filtered, double *d_img);

/* ---- split-Bregman TV: tomography/tv_hpc.F90:162-363 (tvopt) ---------------
 * Solves every slice of f (S*T*N) with ninner x nouter Bregman iterations of
 * ncg CG steps each; writes the TV result to tv_out and the FBP warm start to
 * fbp_out (S*N*N each; fbp_out may be NULL).  Batched: all S slices advance
 * together, CG inner products / step lengths / residual norms in FP64 on the
 * device, the outer iteration replayed as a CUDA graph.
 * acu_tvopt_plain*: the same algorithm as one slice at a time with one kernel
 *   per loop of the reference, direct filter, and the CG scalars read back to
 *   the host every step, as the reference does (the per-slice comparator).  */
int acu_tvopt(acu_ctx *ctx, int nslices, const float *f, int ninner, int nouter, int ncg,
              float lambda, float mu, float *tv_out, float *fbp_out);
int acu_tvopt_dev(acu_ctx *ctx, int nslices, const float *d_f, int ninner, int nouter, int ncg,
                  float lambda, float mu, float *d_tv, float *d_fbp);
int acu_tvopt_plain(acu_ctx *ctx, int nslices, const float *f, int ninner, int nouter, int ncg,
                    float lambda, float mu, float *tv_out, float *fbp_out);
int acu_tvopt_plain_dev(acu_ctx *ctx, int nslices, const float *d_f, int ninner, int nouter,
                        int ncg, float lambda, float mu, float *d_tv, float *d_fbp);
int acu_tvopt_dev_f64(acu_ctx *ctx, int nslices, const double *d_f, int ninner, int nouter,
                      int ncg, double lambda, double mu, double *d_tv, double *d_fbp);
/* The batched solver in steps, for callers that interleave their own work or
 * time the outer iterations: acu_tv_begin = allocation, copy of d_f (S*T*N,
 * device) and the warm start of tv_hpc.F90:172-202 (FBP into d_fbp when not
 * NULL); acu_tv_iterate = nouter more outer iterations of tv_hpc.F90:205-353
 * (callable repeatedly; the iteration is captured once as a CUDA graph);
 * acu_tv_end = copy of the current TV iterate to d_tv (S*N*N, device).
 * acu_tvopt_dev is begin + iterate(nouter) + end.                            */
int acu_tv_begin(acu_ctx *ctx, int nslices, const float *d_f, int ninner, int ncg, float lambda,
                 float mu, float *d_fbp);
int acu_tv_iterate(acu_ctx *ctx, int nouter);
int acu_tv_end(acu_ctx *ctx, float *d_tv);
/* ---- registration-aware TV objective and its gradient (new) -----------------
 * For S slices with per-angle detector offsets off[S][T] (pixels; NULL = 0):
 *   loss[s] = 1/2 |A_off u - y|^2 + lambda * sum_i sqrt((Dx u)_i^2 + eps^2)
 *                                            + sqrt((Dy u)_i^2 + eps^2)
 * A_off is the projector of tv_hpc.F90:137-156 with bin jy read at detector
 * coordinate jy + off[t] (off = 0 is acu_radon exactly); Dx, Dy are the
 * periodic backward differences of the shrinkage step (tv_hpc.F90:305-325).
 * Writes loss (host, S doubles), d_grad_u (S*N*N) = A_off^T r + lambda
 * dTV/du, computed with the exact adjoint, and d_grad_off (S*T) = the
 * derivative with respect to each angle's offset (either may be NULL).     */
int acu_tv_loss_grad_dev(acu_ctx *ctx, int nslices, const float *d_u, const float *d_off, const float *d_y,
                         float lambda, float eps, double *loss, float *d_grad_u, float *d_grad_off);
int acu_tv_loss_grad_dev_f64(acu_ctx *ctx, int nslices, const double *d_u, const double *d_off,
                             const double *d_y, double lambda, double eps, double *loss, double *d_grad_u,
                             double *d_grad_off);
/* Print-only Err_diff of the last outer iteration per slice (tv_hpc.F90:327-333),
 * available after a tvopt call with ACU_OPT_VERBOSE set.                     */
int acu_tv_last_delta(const acu_ctx *ctx, int nslices, double *delta);

/* ---- projection preprocessing (device pointers, ordered on ctx's stream) ----
 * Any context works, including one created with nimage = 0.  Projections are
 * ndet x nrows floats with the detector fastest (the reference's square
 * nimage x nimage projections generalised to ndet != nrows); a stack holds
 * nproj of them.  Angles are host arrays in degrees.
 *
 * acu_frame_average*: tomography/fits_to_hpc.F90:183-210 -- mean of a stack
 *   of open-beam (flat) or dark frames, summed in frame order.
 * acu_normalize*: fits_to_hpc.F90:243 (mode 0: -log(I / max(OB,1)), the
 *   reference's active line) and :244 (mode 1: -log(max(I-DF,1e-16) /
 *   max(OB-DF,1)), its flat/dark alternative), for nproj projections.
 * acu_pick_angle_dev: projections_to_sinogram_hpc.F90:141-224 -- the
 *   projection at exactly `target` degrees (0 or 180): the nearest one when
 *   it lies at the target or has no neighbour across it, else the linear
 *   interpolation of the two projections bracketing the target.
 * acu_register_dev: :231-364 -- centre-of-mass initial shift and the
 *   multiplicative pattern search over (tilt, shift) minimising the mirrored
 *   L1 mismatch of the resampled 0/180-degree projections.  theta in radians,
 *   shift as a fraction of ndet, as the reference.
 * acu_xcorr_register_dev: new -- integer lag k maximising the correlation of
 *   the 0-degree projection with the mirrored 180-degree one over
 *   k = -kmax..kmax (products summed as 2^-32 fixed point, so the integer lag is
 *   bit-exact and independent of summation order; ties go to the lowest k),
 *   and the parabolic sub-pixel vertex k_sub.  The axis sits at detector
 *   position (ndet - 1 + k_sub)/2 (0-based); the equivalent reference shift
 *   is (add - k_sub) / (2 ndet), add = 1 for even ndet.
 * acu_median27_dev: :426-452 -- median of the 3x3 neighbourhood (clamped) in
 *   the previous, current and next projection, with the intended slots 1..27
 *   (the reference's slot expression indexes -2..24).
 * acu_resample_dev: :456-470 -- bilinear resample onto the (ndet+add) x nrows
 *   grid under (theta, shift), with the reference's clamps.
 * acu_proj_to_sino_dev: :397-487 -- median, resample and transpose of every
 *   projection into nrows sinograms of nproj x (ndet+add) (slice-major:
 *   sino[row][projection][det]).
 * acu_proj_to_sino_u16: the whole chain on host buffers: raw uint16
 *   projections, flat and dark stacks -> averages -> normalisation (norm_mode)
 *   -> 0/180 picks -> registration (reg_method 0: the reference's pattern
 *   search, 1: cross-correlation) -> median, resample, transpose.            */
int acu_frame_average_u16_dev(acu_ctx *ctx, int nframes, long npix, const uint16_t *d_frames, float *d_out);
int acu_frame_average_dev(acu_ctx *ctx, int nframes, long npix, const float *d_frames, float *d_out);
int acu_normalize_u16_dev(acu_ctx *ctx, int mode, int nproj, long npix, const uint16_t *d_raw,
                          const float *d_ob, const float *d_df, float *d_out);
int acu_normalize_dev(acu_ctx *ctx, int mode, int nproj, long npix, const float *d_raw, const float *d_ob,
                      const float *d_df, float *d_out);
int acu_pick_angle_dev(acu_ctx *ctx, int nfiles, const float *theta_deg, long npix, const float *d_proj,
                       float target, float *d_out);
int acu_register_dev(acu_ctx *ctx, int ndet, int nrows, const float *d_p0, const float *d_p180,
                     float *theta_out, float *shift_out, int *evals_out);
int acu_xcorr_register_dev(acu_ctx *ctx, int ndet, int nrows, const float *d_p0, const float *d_p180,
                           int kmax, int64_t *corr_out, int *k_best, double *k_sub);
int acu_median27_dev(acu_ctx *ctx, int ndet, int nrows, const float *d_l, const float *d_c, const float *d_r,
                     float *d_out);
int acu_resample_dev(acu_ctx *ctx, int ndet, int nrows, const float *d_src, float theta, float shift,
                     float *d_out);
int acu_proj_to_sino_dev(acu_ctx *ctx, int nproj, int ndet, int nrows, const float *d_proj, float theta,
                         float shift, float *d_sino);
/* Host-buffer forms used by the drivers: normalisation of a uint16 stack with
 * its flat and dark stacks (fits_to_hpc.F90:183-248), and the chain from
 * normalised float projections to sinograms (projections_to_sinogram_hpc.F90). */
int acu_normalize_stack_u16(acu_ctx *ctx, int mode, int nproj, long npix, const uint16_t *raw, int nflat,
                            const uint16_t *flats, int ndark, const uint16_t *darks, float *out);
/* The same normalisation of float projections (the pixel values cfitsio's
 * ftgpve returns in fits_to_hpc.F90:224) given the averaged flat and dark
 * frames (:183-210); df may be null for mode 0. */
int acu_normalize_stack(acu_ctx *ctx, int mode, int nproj, long npix, const float *raw, const float *ob,
                        const float *df, float *out);
int acu_proj_to_sino(acu_ctx *ctx, int nproj, int ndet, int nrows, const float *proj, const float *theta_deg,
                     int reg_method, float *sino_out, float *theta_out, float *shift_out);
int acu_proj_to_sino_u16(acu_ctx *ctx, int nproj, int ndet, int nrows, const uint16_t *raw,
                         const float *theta_deg, int nflat, const uint16_t *flats, int ndark,
                         const uint16_t *darks, int norm_mode, int reg_method, float *sino_out,
                         float *theta_out, float *shift_out);

/* ---- ragged batches: independent problems of different size ----------------
 * nprob problems, problem i with grid side nimage[i], ntheta[i] angles (its
 * angles at theta_concat[sum_{j<i} ntheta[j] ...]) and mask taper wpu[i];
 * each problem is one slice.  acu_batch_tvopt solves all of them with
 * tomography/tv_hpc.F90:162-363 (same ninner/nouter/ncg/lambda/mu), f holding
 * the sinograms back to back (T_i*N_i floats each) and tv / fbp the images
 * (N_i*N_i each), host buffers.  The projector and backprojection run as
 * persistent kernels over (problem, angle, bin block) / (problem, pixel tile)
 * work items, largest problem first, one launch per operator; their block
 * shapes are chosen by timing candidates on the batch at first use
 * (acu_batch_tuning reports the choice).  acu_batch_op runs one operator
 * (op 0: radon, images -> sinograms; op 1: iradon, sinograms -> images).  */
typedef struct acu_batch acu_batch;
int acu_batch_create(acu_batch **batch, int nprob, const int *nimage, const int *ntheta, const float *theta_concat,
                     const int *wpu);
int acu_batch_destroy(acu_batch *batch);
int acu_batch_set_stream(acu_batch *batch, void *cuda_stream);
const char *acu_batch_last_error(const acu_batch *batch);
int acu_batch_tvopt(acu_batch *batch, const float *f, int ninner, int nouter, int ncg, float lambda, float mu,
                    float *tv_out, float *fbp_out);
int acu_batch_op(acu_batch *batch, int op, const float *in, float *out);
int acu_batch_tuning(const acu_batch *batch, int *radon_warps, int *bp_rows);
/* ACU_OPT_POSITIONS (0 or 1, default 1) and ACU_OPT_RADON_REFRESH (default 5) for every
 * problem of the batch; other options are rejected with ACU_ERR_INVALID.  The
 * batch always forms the initial CG residual from one backprojection of
 * fk - radon(uk) (ACU_OPT_RESIDUAL = 1). */
int acu_batch_set_option(acu_batch *batch, int option, int value);

/* ---- cross-correlation registration without device allocation --------------
 * No counterpart in the reference.  Same computation and results as
 * acu_xcorr_register_dev, for callers that must not have the library allocate
 * device memory (device memory reserved up front by an acquisition pipeline
 * or owned by another allocator, or a thread that cannot afford the implicit
 * synchronisation of cudaMalloc/cudaFree).  It needs no context: its scratch
 * is a fixed array inside the library, 2*2048+3 eight-byte words, present on
 * every GPU that loads the library until the process exits, so kmax is
 * limited to 1..2048 (larger kmax returns ACU_ERR_INVALID).  The first call on
 * a device resolves that array's device address (cudaGetSymbolAddress) with
 * the device current; make that first call before any stream capture.  All
 * calls share the one array: each call clears the sums it uses before
 * accumulating, and calls whose work overlaps on the GPU (other streams,
 * other host threads) race on it -- serialise them.  The work is ordered on
 * `stream` (NULL: the legacy default stream); the call returns after the
 * results are read back.  Errors are reported by acu_last_error(NULL).      */
int acu_xcorr_register_noalloc(int ndet, int nrows, const float *d_p0, const float *d_p180, int kmax,
                               int64_t *corr_out, int *k_best, double *k_sub, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* ACUMEN_GPU_H */
