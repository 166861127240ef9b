// Ragged batches of independent problems (different grid sizes and angle
// counts), solved together: one persistent launch per operator, work items
// taken from a device counter (batch.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace acu {

// One problem of a ragged batch.  Offsets are in elements of the
// concatenated arrays; item prefix sums index the work lists.
struct ProbDesc {
    int N, T, L, lg;        // grid side, angles, FFT length and log2
    float mid;              // (N+1)/2 (integer division)
    int nbx;                // 32-bin blocks per angle
    long long img;          // image offset (N*N per problem)
    long long sino;         // sinogram offset (T*N)
    long long sc;           // angle-table offset (2T floats)
    long long cm;           // mask offset (N*N)
    long long fh;           // FFT spectrum offset (L)
    long long it_radon;     // first projector item: T * nbx items per problem
    long long it_bp;        // first backprojection item: ceil(N/32) * ceil(N/8)
    long long it_fft;       // first filter item: ceil(T/2)
    long long it_ew;        // first element-wise block: ceil(N*N / 1024)
    long long it_tr;        // first transpose tile: ceil(N/32)^2
};

struct BatchDev {
    int nprob = 0;
    const ProbDesc* pd = nullptr;
    const float* sc_bp = nullptr;
    const float* sc_fp = nullptr;
    const float4* xsc_bp = nullptr;   // exact-position tables, [angle][4] (index ProbDesc::sc / 2)
    const float4* xsc_fp = nullptr;
    int exact = 1;                    // 1: exact sample positions (default), 0: the reference's (acu_batch_set_option)
    const float* cmask = nullptr;
    const float* fft_h = nullptr;
    const float* fft_h_x = nullptr;   // spectra of the FP64 taps (exact positions)
    const float2* tw = nullptr;   // twiddles of the largest L (Lmax entries)
    int Lmax = 0;
    long long n_radon = 0, n_bp = 0, n_fft = 0, n_ew = 0, n_tr = 0;   // item totals
    float* IT = nullptr;          // work buffer: transposed images (img_total floats)
    long long img_total = 0, sino_total = 0;
    int* counter = nullptr;       // work counters (one per persistent kernel)
    int radon_warps = 4;          // autotuned: warps per projector block
    int bp_rows = 8;              // autotuned: pixel rows per backprojection block
};

void batch_radon(const BatchDev& b, const float* img, float* sino, int slot, cudaStream_t st);
void batch_filter(const BatchDev& b, const float* sino, float* out, cudaStream_t st);
void batch_backproject(const BatchDev& b, const float* q, float* img, int slot, cudaStream_t st);
// element-wise TV steps; per-problem FP64 scalars rsold/alpha/beta/delta[nprob],
// partials part[n_ew]
void batch_rhs(const BatchDev& b, float mu, float lambda, const float* ifkt, const float* dx, const float* bx,
               const float* dy, const float* by, float* rhs, cudaStream_t st);
void batch_resid(const BatchDev& b, float mu, float lambda, const float* rhs, const float* iukt, const float* uk,
                 float* r, float* p, double* part, cudaStream_t st);
void batch_apply(const BatchDev& b, float mu, float lambda, const float* irpt, const float* p, float* Ap,
                 double* part, cudaStream_t st);
void batch_update(const BatchDev& b, const float* p, const float* Ap, float* uk, float* r, const double* alpha,
                  double* part, cudaStream_t st);
void batch_pupdate(const BatchDev& b, const float* r, float* p, const double* beta, cudaStream_t st);
void batch_shrink(const BatchDev& b, float lambda, const float* uk, float* dx, float* bx, float* dy, float* by,
                  cudaStream_t st);
void batch_fk(const BatchDev& b, float* fk, const float* f, const float* ruk, cudaStream_t st);
void batch_diff(const BatchDev& b, const float* a, const float* c, float* out, cudaStream_t st);
void batch_sino_axpy(const BatchDev& b, const double* alpha, const float* x, float* y, cudaStream_t st);
// which: 0 rsold = sum; 1 alpha = rsold / sum; 2 beta = sum / rsold, rsold = sum
void batch_finalize(const BatchDev& b, int which, const double* part, double* rsold, double* alpha, double* beta,
                    cudaStream_t st);

}  // namespace acu
