// Internal definition of the library context shared by the API translation
// units (api.cu, prep.cu, grad.cu, batch.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/acumen_gpu.h"
#include "kernels.h"

namespace acu {

extern thread_local std::string g_last_error;

struct DevBuf {
    void* p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    // grow-only; returns a cudaError_t
    cudaError_t ensure(size_t bytes)
    {
        if (bytes <= n && p) return cudaSuccess;
        release();
        if (bytes == 0) bytes = 16;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e != cudaSuccess) {
            p = nullptr;
            return e;
        }
        n = bytes;
        return cudaSuccess;
    }
    template <typename T>
    T* as() const { return reinterpret_cast<T*>(p); }
};

template <typename Real>
struct GeomSet {
    bool ready = false;
    DevBuf sc_bp, sc_fp, filt, cmask, fft_h, fft_h_x, fft_tw, fft_tw16, fp_order, lines_order, xsc_bp, xsc_fp;
    std::vector<float4> hx_bp;   // host copy of xsc_bp
    std::vector<float4> hs_bp;   // host copy of sc_bp as (sin, cos, 0, 0) (single precision)
    DevGeom<Real> d;
};

// Work buffers of the TV solver for one precision (lane layout, G groups).
template <typename Real>
struct TvState {
    DevBuf f, fk, ruk, rp, q;                                   // T*N per slice
    DevBuf uk, ukp, dx, dy, bx, by, rhs, r, p, Ap, tmp;         // N*N per slice
    // ACU_OPT_RESIDUAL = 2: bd = iradon(f - radon(uk)) and dacc = iradon(fk - f),
    // carried so that iradon(fk - radon(uk)) = bd + dacc needs no backprojection
    DevBuf bd, dacc;                                            // N*N per slice
    bool carried_valid = false;                                 // bd and dacc follow the iterate
    DevBuf rsold, alpha, beta, delta, part;                     // FP64 scalars
    cudaGraphExec_t graph = nullptr;       // one outer iteration (radon(uk) recomputed at its end)
    cudaGraphExec_t graph_inc = nullptr;   // the same with radon(uk) carried by the CG updates only
    std::string graph_key;
    // the active batched problem (acu_tv_begin .. acu_tv_end)
    bool active = false;
    int S = 0, G = 0, V = 1, ninner = 0, ncg = 0, nblk = 0, outer_done = 0;
    double lambda = 0, mu = 0;
    ~TvState()
    {
        if (graph) cudaGraphExecDestroy(graph);
        if (graph_inc) cudaGraphExecDestroy(graph_inc);
    }
};

}  // namespace acu

struct acu_ctx {
    int N = 0, T = 0, wpu = 0;
    std::vector<float> theta;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    int opt_filter = 0;  // FFT ramp filter
    int opt_lanes = 0;
    int opt_graph = 1;
    int opt_verbose = 0;
    int opt_print_every = 50;
    int opt_slice_base = 1;
    int opt_max_batch = 0;   // slices per device batch of the TV solver: 0 as many as fit
    int opt_refresh = 5;     // radon(uk): 1 recomputed every outer iteration (reference), K >= 2 every K-th, 0 never
    int opt_residual = 2;    // initial CG residual: 2 carried backprojections (none per step), 1 one backprojection of fk - radon(uk), 0 two (reference)
    int opt_positions = 1;   // 1 exact positions (default), 0 the reference's single-precision positions
    int opt_projector = 7;   // single-precision projector: 0 pair images, 1 lane image + transpose, 2 row-parity
                             // loads, 3 taps reused, 4 reuse + clipped steps, 5 the same with paired FMAs,
                             // 6 pixel lines, 7 automatic (6 or 5 by how full the 32-slice lines are)
    std::string err;
    acu::GeomSet<float> g32;
    acu::GeomSet<double> g64;
    // operator work buffers
    acu::DevBuf w_in, w_out, w_q, w_host_in, w_host_out;
    acu::DevBuf pairP, pairPT;   // pair images of the single-precision projector
    acu::DevBuf lineL, lineA;    // line image and ray sums of projector variant 6
    acu::DevBuf w_part;          // FP64 / int64 partial sums of the preprocessing reductions
    acu::TvState<float> tv32;
    acu::TvState<double> tv64;
    std::vector<double> last_delta;
};

namespace acu {

int set_err(acu_ctx* ctx, int code, const char* fmt, ...);

#define CK(ctx, call)                                                                           \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess)                                                                  \
            return set_err(ctx, e_ == cudaErrorMemoryAllocation ? ACU_ERR_NOMEM : ACU_ERR_CUDA, \
                           "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

#define CKLAUNCH(ctx) CK(ctx, cudaGetLastError())

#define CKRET(expr)              \
    do {                         \
        int r_ = (expr);         \
        if (r_ != ACU_OK) return r_; \
    } while (0)


}  // namespace acu
