// Element-wise steps of the split-Bregman / CG solver
// (tomography/tv_hpc.F90:187-346) on slice groups in lane layout, the FP64
// per-slice CG scalars, and the plain <-> lane layout conversions.
//
// Every reduction is deterministic: each block writes one FP64 partial per
// slice, and a finaliser sums the partials of a slice in a fixed order.
#include "common.cuh"
#include "kernels.h"

namespace acu {

constexpr int EW_THREADS = 256;
constexpr int EW_MAX_BLOCKS = 512;

static inline int ew_blocks(size_t npix)
{
    size_t b = (npix + EW_THREADS - 1) / EW_THREADS;
    return (int)(b < EW_MAX_BLOCKS ? b : EW_MAX_BLOCKS);
}

// periodic neighbours of tomography/tv_hpc.F90:220-237 in 0-based indices
__device__ __forceinline__ int nb_next(int j, int N) { return j + 1 == N ? 0 : j + 1; }
__device__ __forceinline__ int nb_prev(int j, int N) { return j == 0 ? N - 1 : j - 1; }

template <typename Real, int V>
__device__ __forceinline__ void write_partials(const SumAcc<Real> (&part)[V], double* out, int nblk)
{
    __shared__ double sh[32];
    const int g = blockIdx.y;
#pragma unroll
    for (int v = 0; v < V; ++v) {
        double r = block_sum(part[v].value(), sh);
        if (threadIdx.x == 0) out[(size_t)(g * V + v) * nblk + blockIdx.x] = r;
    }
}

// ---- rhs = mu*ifkt + lambda*(d - b terms)  (tv_hpc.F90:217-225) ------------
template <typename Real, int V>
__global__ void __launch_bounds__(EW_THREADS) k_rhs(int N, Real mu, Real lambda, const Real* __restrict__ ifkt,
                                                    const Real* __restrict__ dx, const Real* __restrict__ bx,
                                                    const Real* __restrict__ dy, const Real* __restrict__ by,
                                                    Real* __restrict__ rhs, const Real* __restrict__ ifkt2)
{
    const size_t NN = (size_t)N * N;
    const size_t base = (size_t)blockIdx.y * NN * V;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < NN; i += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % N), y = (int)(i / N);
        const size_t ixn = ((size_t)y * N + nb_next(x, N)) * V + base;
        const size_t iyn = ((size_t)nb_next(y, N) * N + x) * V + base;
        const size_t ii = i * V + base;
        Lanes<Real, V> a = ld_lanes_rw<Real, V>(ifkt + ii);
        if (ifkt2) {
            const Lanes<Real, V> a2 = ld_lanes_rw<Real, V>(ifkt2 + ii);
#pragma unroll
            for (int v = 0; v < V; ++v) a.v[v] = a.v[v] + a2.v[v];
        }
        Lanes<Real, V> dxn = ld_lanes_rw<Real, V>(dx + ixn), bxn = ld_lanes_rw<Real, V>(bx + ixn);
        Lanes<Real, V> dx0 = ld_lanes_rw<Real, V>(dx + ii), bx0 = ld_lanes_rw<Real, V>(bx + ii);
        Lanes<Real, V> dyn = ld_lanes_rw<Real, V>(dy + iyn), byn = ld_lanes_rw<Real, V>(by + iyn);
        Lanes<Real, V> dy0 = ld_lanes_rw<Real, V>(dy + ii), by0 = ld_lanes_rw<Real, V>(by + ii);
        Lanes<Real, V> o;
#pragma unroll
        for (int v = 0; v < V; ++v) {
            Real acc = dxn.v[v] - bxn.v[v];
            acc = acc - dx0.v[v];
            acc = acc + bx0.v[v];
            acc = acc + dyn.v[v];
            acc = acc - byn.v[v];
            acc = acc - dy0.v[v];
            acc = acc + by0.v[v];
            o.v[v] = mu * a.v[v] + lambda * acc;
        }
        st_lanes<Real, V>(rhs + ii, o);
    }
}

template <typename Real, int V>
__device__ __forceinline__ Lanes<Real, V> lap5(const Real* u, int N, int x, int y, size_t base)
{
    const Lanes<Real, V> c = ld_lanes_rw<Real, V>(u + base + ((size_t)y * N + x) * V);
    const Lanes<Real, V> xl = ld_lanes_rw<Real, V>(u + base + ((size_t)y * N + nb_prev(x, N)) * V);
    const Lanes<Real, V> xr = ld_lanes_rw<Real, V>(u + base + ((size_t)y * N + nb_next(x, N)) * V);
    const Lanes<Real, V> yl = ld_lanes_rw<Real, V>(u + base + ((size_t)nb_prev(y, N) * N + x) * V);
    const Lanes<Real, V> yr = ld_lanes_rw<Real, V>(u + base + ((size_t)nb_next(y, N) * N + x) * V);
    Lanes<Real, V> o;
#pragma unroll
    for (int v = 0; v < V; ++v) o.v[v] = (((Real(4) * c.v[v] - xl.v[v]) - xr.v[v]) - yl.v[v]) - yr.v[v];
    return o;
}

// ---- r = rhs - mu*iukt - lambda*Lap(uk); p = r; rsold = sum r^2 (:231-249) --
template <typename Real, int V>
__global__ void __launch_bounds__(EW_THREADS) k_resid(int N, Real mu, Real lambda, const Real* __restrict__ rhs,
                                                      const Real* __restrict__ iukt, const Real* __restrict__ uk,
                                                      Real* __restrict__ r, Real* __restrict__ p, double* part,
                                                      int nblk)
{
    const size_t NN = (size_t)N * N;
    const size_t base = (size_t)blockIdx.y * NN * V;
    SumAcc<Real> acc[V];
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < NN; i += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % N), y = (int)(i / N);
        const size_t ii = i * V + base;
        const Lanes<Real, V> L = lap5<Real, V>(uk, N, x, y, base);
        const Lanes<Real, V> h = ld_lanes_rw<Real, V>(rhs + ii);
        Lanes<Real, V> a;   // iukt == nullptr: rhs already holds mu * iradon(fk - radon(uk))
        if (iukt)
            a = ld_lanes_rw<Real, V>(iukt + ii);
        else
#pragma unroll
            for (int v = 0; v < V; ++v) a.v[v] = Real(0);
        Lanes<Real, V> o;
#pragma unroll
        for (int v = 0; v < V; ++v) {
            o.v[v] = (h.v[v] - mu * a.v[v]) - lambda * L.v[v];
            acc[v].add_prod(o.v[v], o.v[v]);
        }
        st_lanes<Real, V>(r + ii, o);
        st_lanes<Real, V>(p + ii, o);
    }
    write_partials<Real, V>(acc, part, nblk);
}

// ---- Ap = mu*irpt + lambda*Lap(p); num = sum p*Ap  (:257-274) ---------------
template <typename Real, int V>
__global__ void __launch_bounds__(EW_THREADS) k_apply(int N, Real mu, Real lambda, const Real* __restrict__ irpt,
                                                      const Real* __restrict__ p, Real* __restrict__ Ap,
                                                      double* part, int nblk)
{
    const size_t NN = (size_t)N * N;
    const size_t base = (size_t)blockIdx.y * NN * V;
    SumAcc<Real> acc[V];
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < NN; i += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % N), y = (int)(i / N);
        const size_t ii = i * V + base;
        const Lanes<Real, V> L = lap5<Real, V>(p, N, x, y, base);
        const Lanes<Real, V> a = ld_lanes_rw<Real, V>(irpt + ii);
        const Lanes<Real, V> pc = ld_lanes_rw<Real, V>(p + ii);
        Lanes<Real, V> o;
#pragma unroll
        for (int v = 0; v < V; ++v) {
            o.v[v] = mu * a.v[v] + lambda * L.v[v];
            acc[v].add_prod(pc.v[v], o.v[v]);
        }
        st_lanes<Real, V>(Ap + ii, o);
    }
    write_partials<Real, V>(acc, part, nblk);
}

// ---- uk += alpha p; r -= alpha Ap; rsnew = sum r^2  (:277-292) -------------
template <typename Real, int V>
__global__ void __launch_bounds__(EW_THREADS) k_update(int N, const Real* __restrict__ p, const Real* __restrict__ Ap,
                                                       Real* __restrict__ uk, Real* __restrict__ r,
                                                       const double* __restrict__ alpha, double* part, int nblk,
                                                       const Real* __restrict__ irpt, Real* __restrict__ bd)
{
    const size_t NN = (size_t)N * N;
    const int g = blockIdx.y;
    const size_t base = (size_t)g * NN * V;
    Real al[V];
#pragma unroll
    for (int v = 0; v < V; ++v) al[v] = (Real)alpha[g * V + v];
    SumAcc<Real> acc[V];
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < NN; i += (size_t)gridDim.x * blockDim.x) {
        const size_t ii = i * V + base;
        Lanes<Real, V> u = ld_lanes_rw<Real, V>(uk + ii), rr = ld_lanes_rw<Real, V>(r + ii);
        const Lanes<Real, V> pp = ld_lanes_rw<Real, V>(p + ii), aa = ld_lanes_rw<Real, V>(Ap + ii);
#pragma unroll
        for (int v = 0; v < V; ++v) {
            u.v[v] = u.v[v] + al[v] * pp.v[v];
            rr.v[v] = rr.v[v] - al[v] * aa.v[v];
            acc[v].add_prod(rr.v[v], rr.v[v]);
        }
        st_lanes<Real, V>(uk + ii, u);
        st_lanes<Real, V>(r + ii, rr);
        if (bd) {   // iradon(f - radon(uk)) follows uk += alpha p
            Lanes<Real, V> b = ld_lanes_rw<Real, V>(bd + ii);
            const Lanes<Real, V> t = ld_lanes_rw<Real, V>(irpt + ii);
#pragma unroll
            for (int v = 0; v < V; ++v) b.v[v] = b.v[v] - al[v] * t.v[v];
            st_lanes<Real, V>(bd + ii, b);
        }
    }
    write_partials<Real, V>(acc, part, nblk);
}

// ---- p = r + (rsnew/rsold) p  (:294-299) -------------------------------------
template <typename Real, int V>
__global__ void __launch_bounds__(EW_THREADS) k_pupdate(int N, const Real* __restrict__ r, Real* __restrict__ p,
                                                        const double* __restrict__ beta)
{
    const size_t NN = (size_t)N * N;
    const int g = blockIdx.y;
    const size_t base = (size_t)g * NN * V;
    Real be[V];
#pragma unroll
    for (int v = 0; v < V; ++v) be[v] = (Real)beta[g * V + v];
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < NN; i += (size_t)gridDim.x * blockDim.x) {
        const size_t ii = i * V + base;
        const Lanes<Real, V> rr = ld_lanes_rw<Real, V>(r + ii);
        Lanes<Real, V> pp = ld_lanes_rw<Real, V>(p + ii);
#pragma unroll
        for (int v = 0; v < V; ++v) pp.v[v] = rr.v[v] + be[v] * pp.v[v];
        st_lanes<Real, V>(p + ii, pp);
    }
}

// ---- shrinkage (:305-325) and the print-only Err_diff (:327-333) ------------
template <typename Real>
__device__ __forceinline__ Real shrink1(Real t, Real thr)
{
    if (t == Real(0)) return Real(0);
    const Real a = t < Real(0) ? -t : t;
    const Real m = (a - thr) > Real(0) ? (a - thr) : Real(0);
    return (m * t) / a;
}

template <typename Real, int V>
__global__ void __launch_bounds__(EW_THREADS) k_shrink(int N, Real lambda, const Real* __restrict__ uk,
                                                       Real* __restrict__ dx, Real* __restrict__ bx,
                                                       Real* __restrict__ dy, Real* __restrict__ by,
                                                       const Real* __restrict__ ukp, double* part, int nblk)
{
    const size_t NN = (size_t)N * N;
    const size_t base = (size_t)blockIdx.y * NN * V;
    const Real thr = Real(1) / lambda;
    SumAcc<Real> acc[V];
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < NN; i += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(i % N), y = (int)(i / N);
        const size_t ii = i * V + base;
        const Lanes<Real, V> u = ld_lanes_rw<Real, V>(uk + ii);
        const Lanes<Real, V> uxl = ld_lanes_rw<Real, V>(uk + base + ((size_t)y * N + nb_prev(x, N)) * V);
        const Lanes<Real, V> uyl = ld_lanes_rw<Real, V>(uk + base + ((size_t)nb_prev(y, N) * N + x) * V);
        const Lanes<Real, V> b0 = ld_lanes_rw<Real, V>(bx + ii), b1 = ld_lanes_rw<Real, V>(by + ii);
        Lanes<Real, V> ox, obx, oy, oby;
#pragma unroll
        for (int v = 0; v < V; ++v) {
            Real t = (uxl.v[v] - u.v[v]) + b0.v[v];
            ox.v[v] = shrink1(t, thr);
            obx.v[v] = t - ox.v[v];
            t = (b1.v[v] + uyl.v[v]) - u.v[v];
            oy.v[v] = shrink1(t, thr);
            oby.v[v] = t - oy.v[v];
        }
        st_lanes<Real, V>(dx + ii, ox);
        st_lanes<Real, V>(bx + ii, obx);
        st_lanes<Real, V>(dy + ii, oy);
        st_lanes<Real, V>(by + ii, oby);
        if (ukp) {
            const Lanes<Real, V> q = ld_lanes_rw<Real, V>(ukp + ii);
#pragma unroll
            for (int v = 0; v < V; ++v) {
                const Real d = u.v[v] - q.v[v];
                acc[v].add(d < Real(0) ? -d : d);
            }
        }
    }
    if (ukp) write_partials<Real, V>(acc, part, nblk);
}

// ---- fk = fk + f - radon(uk)  (:341-346) -------------------------------------
template <typename Real>
__global__ void k_fk(size_t n, Real* __restrict__ fk, const Real* __restrict__ f, const Real* __restrict__ ruk)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        fk[i] = (fk[i] + f[i]) - ruk[i];
}

// ---- FP64 finalisers ---------------------------------------------------------
__global__ void k_cg_finalize(int which, const double* __restrict__ part, int nblk, double* rsold,
                              double* alpha, double* beta, double* delta)
{
    __shared__ double sh[32];
    const int s = blockIdx.x;
    double v = 0.0;
    for (int i = threadIdx.x; i < nblk; i += blockDim.x) v += part[(size_t)s * nblk + i];
    const double sum = block_sum(v, sh);
    if (threadIdx.x == 0) {
        if (which == 0) {
            rsold[s] = sum;
        } else if (which == 1) {
            alpha[s] = (sum != 0.0) ? rsold[s] / sum : 0.0;
        } else if (which == 2) {
            beta[s] = (rsold[s] != 0.0) ? sum / rsold[s] : 0.0;
            rsold[s] = sum;
        } else {
            delta[s] = sum;
        }
    }
}

void launch_cg_finalize(int which, int S, const TvScalars& sc, cudaStream_t st)
{
    k_cg_finalize<<<S, 256, 0, st>>>(which, sc.part, sc.nblk, sc.rsold, sc.alpha, sc.beta, sc.delta);
}

template <typename Real, int V>
void TvEw<Real, V>::rhs(int N, int G, Real mu, Real lambda, const Real* ifkt, const Real* dx, const Real* bx,
                        const Real* dy, const Real* by, Real* out, cudaStream_t st, const Real* ifkt2)
{
    dim3 grd(ew_blocks((size_t)N * N), G);
    k_rhs<Real, V><<<grd, EW_THREADS, 0, st>>>(N, mu, lambda, ifkt, dx, bx, dy, by, out, ifkt2);
}
template <typename Real, int V>
void TvEw<Real, V>::resid(int N, int G, Real mu, Real lambda, const Real* rhs, const Real* iukt, const Real* uk,
                          Real* r, Real* p, const TvScalars& sc, cudaStream_t st)
{
    dim3 grd(sc.nblk, G);
    k_resid<Real, V><<<grd, EW_THREADS, 0, st>>>(N, mu, lambda, rhs, iukt, uk, r, p, sc.part, sc.nblk);
}
template <typename Real, int V>
void TvEw<Real, V>::apply(int N, int G, Real mu, Real lambda, const Real* irpt, const Real* p, Real* Ap,
                          const TvScalars& sc, cudaStream_t st)
{
    dim3 grd(sc.nblk, G);
    k_apply<Real, V><<<grd, EW_THREADS, 0, st>>>(N, mu, lambda, irpt, p, Ap, sc.part, sc.nblk);
}
template <typename Real, int V>
void TvEw<Real, V>::update(int N, int G, const Real* p, const Real* Ap, Real* uk, Real* r, const TvScalars& sc,
                           cudaStream_t st, const Real* irpt, Real* bd)
{
    dim3 grd(sc.nblk, G);
    k_update<Real, V><<<grd, EW_THREADS, 0, st>>>(N, p, Ap, uk, r, sc.alpha, sc.part, sc.nblk, irpt, bd);
}
template <typename Real, int V>
void TvEw<Real, V>::pupdate(int N, int G, const Real* r, Real* p, const TvScalars& sc, cudaStream_t st)
{
    dim3 grd(sc.nblk, G);
    k_pupdate<Real, V><<<grd, EW_THREADS, 0, st>>>(N, r, p, sc.beta);
}
template <typename Real, int V>
void TvEw<Real, V>::shrink(int N, int G, Real lambda, const Real* uk, Real* dx, Real* bx, Real* dy, Real* by,
                           const Real* ukp, const TvScalars& sc, cudaStream_t st)
{
    dim3 grd(sc.nblk, G);
    k_shrink<Real, V><<<grd, EW_THREADS, 0, st>>>(N, lambda, uk, dx, bx, dy, by, ukp, sc.part, sc.nblk);
}
template <typename Real, int V>
void TvEw<Real, V>::fk_update(size_t n, Real* fk, const Real* f, const Real* ruk, cudaStream_t st)
{
    size_t b = (n + 255) / 256;
    k_fk<Real><<<(unsigned)(b < 4096 ? b : 4096), 256, 0, st>>>(n, fk, f, ruk);
}
// radon(uk + alpha p) = radon(uk) + alpha radon(p): the projection of the
// iterate follows the CG update without a projector launch.
template <typename Real, int V>
__global__ void __launch_bounds__(EW_THREADS) k_sino_axpy(size_t npos, const double* __restrict__ alpha,
                                                          const Real* __restrict__ x, Real* __restrict__ y)
{
    const int g = blockIdx.y;
    Real al[V];
#pragma unroll
    for (int v = 0; v < V; ++v) al[v] = (Real)alpha[g * V + v];
    const size_t base = (size_t)g * npos * V;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < npos; i += (size_t)gridDim.x * blockDim.x) {
        const size_t ii = base + i * V;
        Lanes<Real, V> yy = ld_lanes_rw<Real, V>(y + ii);
        const Lanes<Real, V> xx = ld_lanes_rw<Real, V>(x + ii);
#pragma unroll
        for (int v = 0; v < V; ++v) yy.v[v] = yy.v[v] + al[v] * xx.v[v];
        st_lanes<Real, V>(y + ii, yy);
    }
}
template <typename Real, int V>
void TvEw<Real, V>::sino_axpy(int T, int N, int G, const Real* x, Real* y, const TvScalars& sc, cudaStream_t st)
{
    dim3 grd(sc.nblk, G);
    k_sino_axpy<Real, V><<<grd, EW_THREADS, 0, st>>>((size_t)T * N, sc.alpha, x, y);
}

template <typename Real>
__global__ void k_diff(size_t n, const Real* __restrict__ a, const Real* __restrict__ b, Real* __restrict__ out)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = a[i] - b[i];
}
template <typename Real, int V>
void TvEw<Real, V>::diff(size_t n, const Real* a, const Real* b, Real* out, cudaStream_t st)
{
    size_t nb = (n + 255) / 256;
    k_diff<Real><<<(unsigned)(nb < 4096 ? nb : 4096), 256, 0, st>>>(n, a, b, out);
}

template <typename Real>
__global__ void k_add(size_t n, const Real* __restrict__ x, Real* __restrict__ y)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        y[i] = y[i] + x[i];
}
template <typename Real, int V>
void TvEw<Real, V>::add(size_t n, const Real* x, Real* y, cudaStream_t st)
{
    size_t nb = (n + 255) / 256;
    k_add<Real><<<(unsigned)(nb < 4096 ? nb : 4096), 256, 0, st>>>(n, x, y);
}

// ---- layout conversion -------------------------------------------------------
template <typename Real, int V>
__global__ void k_to_lanes(const Real* __restrict__ plain, Real* __restrict__ lanes, int S, size_t npos)
{
    const int g = blockIdx.y;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < npos; i += (size_t)gridDim.x * blockDim.x) {
        Lanes<Real, V> o;
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const int s = g * V + v;
            o.v[v] = s < S ? plain[(size_t)s * npos + i] : Real(0);
        }
        st_lanes<Real, V>(lanes + ((size_t)g * npos + i) * V, o);
    }
}
template <typename Real, int V>
__global__ void k_from_lanes(const Real* __restrict__ lanes, Real* __restrict__ plain, int S, size_t npos)
{
    const int g = blockIdx.y;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < npos; i += (size_t)gridDim.x * blockDim.x) {
        const Lanes<Real, V> o = ld_lanes_rw<Real, V>(lanes + ((size_t)g * npos + i) * V);
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const int s = g * V + v;
            if (s < S) plain[(size_t)s * npos + i] = o.v[v];
        }
    }
}
template <typename Real, int V>
void launch_to_lanes(const Real* plain, Real* lanes, int S, size_t npos, cudaStream_t st)
{
    const int G = (S + V - 1) / V;
    size_t b = (npos + 255) / 256;
    dim3 grd((unsigned)(b < 2048 ? b : 2048), G);
    k_to_lanes<Real, V><<<grd, 256, 0, st>>>(plain, lanes, S, npos);
}
template <typename Real, int V>
void launch_from_lanes(const Real* lanes, Real* plain, int S, size_t npos, cudaStream_t st)
{
    const int G = (S + V - 1) / V;
    size_t b = (npos + 255) / 256;
    dim3 grd((unsigned)(b < 2048 ? b : 2048), G);
    k_from_lanes<Real, V><<<grd, 256, 0, st>>>(lanes, plain, S, npos);
}

template struct TvEw<float, 1>;
template struct TvEw<float, 4>;
template struct TvEw<double, 1>;
template void launch_to_lanes<float, 4>(const float*, float*, int, size_t, cudaStream_t);
template void launch_from_lanes<float, 4>(const float*, float*, int, size_t, cudaStream_t);

}  // namespace acu
