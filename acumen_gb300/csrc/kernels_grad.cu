// Element-wise and reduction steps of the registration-aware TV objective
//   loss = 1/2 |A_off u - y|^2 + lambda * sum_i [ sqrt((Dx u)_i^2 + eps^2) + sqrt((Dy u)_i^2 + eps^2) ]
// with the periodic backward differences of the reference's shrinkage step
// (tomography/tv_hpc.F90:305-325): (Dx u)(jx,jy) = u(jx-1,jy) - u(jx,jy).
// All sums are FP64 block partials summed in a fixed order.
#include "common.cuh"
#include "kernels.h"

namespace acu {

template <typename Real>
__global__ void __launch_bounds__(256) k_residual(size_t n_per, Real* __restrict__ r, const Real* __restrict__ y,
                                                  double* __restrict__ part, int nblk)
{
    __shared__ double sh[32];
    const int s = blockIdx.y;
    Real* rs = r + (size_t)s * n_per;
    const Real* ys = y + (size_t)s * n_per;
    double acc = 0.0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n_per; i += (size_t)gridDim.x * blockDim.x) {
        const Real v = rs[i] - ys[i];
        rs[i] = v;
        acc += 0.5 * (double)v * (double)v;
    }
    const double t = block_sum(acc, sh);
    if (threadIdx.x == 0) part[(size_t)s * nblk + blockIdx.x] = t;
}

template <typename Real>
__device__ __forceinline__ Real tv_term(Real g, Real eps)
{
    return sqrt(g * g + eps * eps);
}

template <typename Real>
__global__ void __launch_bounds__(256) k_tv_grad(int N, Real lambda, Real eps, const Real* __restrict__ u,
                                                 Real* __restrict__ grad, double* __restrict__ part, int nblk)
{
    __shared__ double sh[32];
    const int s = blockIdx.y;
    const size_t NN = (size_t)N * N;
    const Real* us = u + (size_t)s * NN;
    Real* gs = grad + (size_t)s * NN;
    double acc = 0.0;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < NN; i += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % N), y = (int)(i / N);
        const int xp = x == 0 ? N - 1 : x - 1, xn = x == N - 1 ? 0 : x + 1;
        const int yp = y == 0 ? N - 1 : y - 1, yn = y == N - 1 ? 0 : y + 1;
        const Real c = us[i];
        // terms owned by pixel i: Dx at i and Dy at i
        const Real gx = us[(size_t)y * N + xp] - c, gy = us[(size_t)yp * N + x] - c;
        const Real nx = tv_term(gx, eps), ny = tv_term(gy, eps);
        acc += (double)lambda * ((double)nx + (double)ny);
        // terms of the right / lower neighbour that contain u_i with a + sign
        const Real gxn = c - us[(size_t)y * N + xn], gyn = c - us[(size_t)yn * N + x];
        const Real nxn = tv_term(gxn, eps), nyn = tv_term(gyn, eps);
        gs[i] += lambda * (-gx / nx - gy / ny + gxn / nxn + gyn / nyn);
    }
    const double t = block_sum(acc, sh);
    if (threadIdx.x == 0) part[(size_t)s * nblk + blockIdx.x] = t;
}

// one block per (angle, slice): grad_off = sum over bins of r * D (FP64)
template <typename Real>
__global__ void __launch_bounds__(256) k_off_grad(int N, int T, const Real* __restrict__ r, const Real* __restrict__ D,
                                                  Real* __restrict__ grad_off)
{
    __shared__ double sh[32];
    const int t = blockIdx.x, s = blockIdx.y;
    const size_t o = ((size_t)s * T + t) * N;
    double acc = 0.0;
    for (int j = threadIdx.x; j < N; j += blockDim.x) acc += (double)r[o + j] * (double)D[o + j];
    const double v = block_sum(acc, sh);
    if (threadIdx.x == 0) grad_off[(size_t)s * T + t] = (Real)v;
}

__global__ void k_sum_rows(const double* __restrict__ part, int nblk, double* __restrict__ out)
{
    __shared__ double sh[32];
    const int s = blockIdx.x;
    double v = 0.0;
    for (int i = threadIdx.x; i < nblk; i += blockDim.x) v += part[(size_t)s * nblk + i];
    const double r = block_sum(v, sh);
    if (threadIdx.x == 0) out[s] = r;
}

template <typename Real>
void GradEw<Real>::residual(size_t n_per, int S, Real* r, const Real* y, double* part, int nblk, cudaStream_t st)
{
    k_residual<Real><<<dim3(nblk, S), 256, 0, st>>>(n_per, r, y, part, nblk);
}
template <typename Real>
void GradEw<Real>::tv_grad(int N, int S, Real lambda, Real eps, const Real* u, Real* grad, double* part, int nblk,
                           cudaStream_t st)
{
    k_tv_grad<Real><<<dim3(nblk, S), 256, 0, st>>>(N, lambda, eps, u, grad, part, nblk);
}
template <typename Real>
void GradEw<Real>::off_grad(int N, int T, int S, const Real* r, const Real* D, Real* grad_off, cudaStream_t st)
{
    k_off_grad<Real><<<dim3(T, S), 256, 0, st>>>(N, T, r, D, grad_off);
}
void launch_sum_rows(const double* part, int rows, int nblk, double* out, cudaStream_t st)
{
    k_sum_rows<<<rows, 256, 0, st>>>(part, nblk, out);
}

template struct GradEw<float>;
template struct GradEw<double>;

}  // namespace acu
