// FFT form of iradon's ramp filter (tomography/tv_hpc.F90:93-105).
//
// The reference convolves every sinogram column directly with the 2N+1 taps
// (O(N^2) per column).  Here each block packs two real columns into one
// complex signal z = a + i b, zero-pads it to L >= 2N-2 (a power of two),
// and computes y = IFFT(H . FFT(z)) with H the real spectrum of the wrapped,
// symmetric tap sequence (computed in double on the host, 1/L folded in).
// Because H is real, Re(y) and Im(y) are the two filtered columns.  At
// L = 4096 in single precision (grids 1449 to 2049) the transforms are three
// radix-16 passes held in registers (k_filter_fft4096); otherwise radix-4
// Stockham stages (a radix-2 stage last when log2 L is odd) in shared memory.
// All twiddles come from double-precision-built tables.
#include "common.cuh"
#include "kernels.h"

namespace acu {

template <typename Real>
struct Cplx;
template <>
struct Cplx<float> {
    using T = float2;
};
template <>
struct Cplx<double> {
    using T = double2;
};

template <typename C>
__device__ __forceinline__ C cmul(C a, C b)
{
    C r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}
template <typename C>
__device__ __forceinline__ C cadd(C a, C b)
{
    C r;
    r.x = a.x + b.x;
    r.y = a.y + b.y;
    return r;
}
template <typename C>
__device__ __forceinline__ C csub(C a, C b)
{
    C r;
    r.x = a.x - b.x;
    r.y = a.y - b.y;
    return r;
}

// Forward DFT of length L (power of two >= 16) held in d0; returns the buffer
// holding the natural-order result (d0 or d1).
// Ns and L are powers of two: indices are formed with shifts and masks.
template <typename C>
__device__ C* fft_stockham(C* d0, C* d1, const C* __restrict__ tw, int L)
{
    const int lgL = 31 - __clz(L);
    for (int Ns = 1, lgNs = 0; Ns < L;) {
        const int R = ((lgL - lgNs) >= 2) ? 4 : 2;
        const int lgR = R == 4 ? 2 : 1;
        const int stride = L >> (lgNs + lgR);
        const int nb = L >> lgR;
        for (int j = threadIdx.x; j < nb; j += blockDim.x) {
            const int k = j & (Ns - 1);
            const int idxD = ((j >> lgNs) << (lgNs + lgR)) + k;
            if (R == 4) {
                C v0 = d0[j];
                C v1 = cmul(d0[j + nb], tw[k * stride]);
                C v2 = cmul(d0[j + 2 * nb], tw[2 * k * stride]);
                C v3 = cmul(d0[j + 3 * nb], tw[3 * k * stride]);
                C a = cadd(v0, v2), b = csub(v0, v2), c = cadd(v1, v3), e = csub(v1, v3);
                C d;               // e * (-i)
                d.x = e.y;
                d.y = -e.x;
                d1[idxD] = cadd(a, c);
                d1[idxD + Ns] = cadd(b, d);
                d1[idxD + 2 * Ns] = csub(a, c);
                d1[idxD + 3 * Ns] = csub(b, d);
            } else {
                C v0 = d0[j];
                C v1 = cmul(d0[j + nb], tw[k * stride]);
                d1[idxD] = cadd(v0, v1);
                d1[idxD + Ns] = csub(v0, v1);
            }
        }
        __syncthreads();
        C* t = d0;
        d0 = d1;
        d1 = t;
        Ns <<= lgR;
        lgNs += lgR;
    }
    return d0;
}

// One block filters two real columns: (a, b) with element n at a[n*stride],
// b[n*stride] (b may be null: treated as zero and not written).
template <typename Real>
__global__ void __launch_bounds__(512) k_filter_fft(const Real* __restrict__ sino, Real* __restrict__ out,
                                                    const Real* __restrict__ H,
                                                    const typename Cplx<Real>::T* __restrict__ tw, int N, int T,
                                                    int L, int V)
{
    using C = typename Cplx<Real>::T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* d0 = reinterpret_cast<C*>(smem_raw);
    C* d1 = d0 + L;
    const int g = blockIdx.y;
    size_t offa, offb;
    int stride;
    bool has_b = true;
    if (V == 4) {
        const int t = blockIdx.x >> 1, h = blockIdx.x & 1;
        offa = (((size_t)g * T + t) * N) * 4 + 2 * h;
        offb = offa + 1;
        stride = 4;
    } else {
        const int t0 = 2 * blockIdx.x;
        offa = ((size_t)g * T + t0) * N;
        offb = offa + N;
        stride = 1;
        has_b = (t0 + 1) < T;
    }
    // 4-slice lanes: the two columns of a half-lane sit side by side (8 or 16
    // bytes, aligned), so they move as one vector
    for (int n = threadIdx.x; n < L; n += blockDim.x) {
        C z;
        if (V == 4) {
            z = n < N ? __ldg(reinterpret_cast<const C*>(sino + offa + (size_t)n * 4)) : C{Real(0), Real(0)};
        } else {
            z.x = n < N ? sino[offa + (size_t)n * stride] : Real(0);
            z.y = (n < N && has_b) ? sino[offb + (size_t)n * stride] : Real(0);
        }
        d0[n] = z;
    }
    __syncthreads();
    C* res = fft_stockham<C>(d0, d1, tw, L);
    C* other = (res == d0) ? d1 : d0;
    // W = H/L * conj(Z); y = conj(FFT(W))
    for (int m = threadIdx.x; m < L; m += blockDim.x) {
        C z = res[m];
        const Real h = H[m];
        C w;
        w.x = h * z.x;
        w.y = -h * z.y;
        res[m] = w;
    }
    __syncthreads();
    C* y = fft_stockham<C>(res, other, tw, L);
    for (int n = threadIdx.x; n < N; n += blockDim.x) {
        const C v = y[n];
        if (V == 4) {
            *reinterpret_cast<C*>(out + offa + (size_t)n * 4) = C{v.x, -v.y};
        } else {
            out[offa + (size_t)n * stride] = v.x;
            if (has_b) out[offb + (size_t)n * stride] = -v.y;
        }
    }
}

// ---- L = 4096 in single precision: three radix-16 passes in registers ------
// Each of 256 threads holds 16 values of a pass: it reads them from the shared
// buffer (element j + 256 m), multiplies by the pass's twiddles, forms a
// 16-point DFT as 4 x 4 (4-point DFTs, the internal twiddles w16^(m1 q2), 4-point
// DFTs) and writes the outputs to their Stockham places.  Against the radix-4
// stages this halves the shared-memory traffic and reads the twiddles from
// tables laid out per pass, which the filter's L1 data pipe (93 % busy with
// the radix-4 stages) needs.  One buffer per transform, padded by one slot per
// 16 so that the strided writes of the first pass spread over the banks.
__device__ __forceinline__ int pad16(int i) { return i + (i >> 4); }

// (a0..a3) -> their 4-point DFT, e^(-2 pi i / 4) = -i
__device__ __forceinline__ void dft4(float2& a0, float2& a1, float2& a2, float2& a3)
{
    const float2 t0 = cadd(a0, a2), t1 = csub(a0, a2), t2 = cadd(a1, a3), e = csub(a1, a3);
    const float2 t3 = make_float2(e.y, -e.x);   // e * (-i)
    a0 = cadd(t0, t2);
    a1 = cadd(t1, t3);
    a2 = csub(t0, t2);
    a3 = csub(t1, t3);
}

// x -> its 16-point DFT y, y[q2 + 4 q1] = sum_m x[m] w16^(m (q2 + 4 q1)),
// m = m1 + 4 m2; the result is returned in x in natural order
__device__ __forceinline__ void dft16(float2 (&x)[16])
{
    constexpr float C8 = 0.92387953251128675613f;   // cos(pi/8)
    constexpr float S8 = 0.38268343236508977173f;   // sin(pi/8)
    constexpr float R2 = 0.70710678118654752440f;   // sqrt(1/2)
#pragma unroll
    for (int m1 = 0; m1 < 4; ++m1) dft4(x[m1], x[m1 + 4], x[m1 + 8], x[m1 + 12]);   // over m2 -> q2 = 0..3
    // x[m1 + 4 q2] *= w16^(m1 q2)
    x[5] = cmul(x[5], make_float2(C8, -S8));     // 1
    x[9] = cmul(x[9], make_float2(R2, -R2));     // 2
    x[13] = cmul(x[13], make_float2(S8, -C8));   // 3
    x[6] = cmul(x[6], make_float2(R2, -R2));     // 2
    x[10] = make_float2(x[10].y, -x[10].x);      // 4: -i
    x[14] = cmul(x[14], make_float2(-R2, -R2));  // 6
    x[7] = cmul(x[7], make_float2(S8, -C8));     // 3
    x[11] = cmul(x[11], make_float2(-R2, -R2));  // 6
    x[15] = cmul(x[15], make_float2(-C8, S8));   // 9
#pragma unroll
    for (int q2 = 0; q2 < 4; ++q2) dft4(x[4 * q2], x[4 * q2 + 1], x[4 * q2 + 2], x[4 * q2 + 3]);   // over m1 -> q1
    // now x[4 q2 + q1] holds y[q2 + 4 q1]: transpose the 4 x 4 index
    float2 y[16];
#pragma unroll
    for (int q2 = 0; q2 < 4; ++q2)
#pragma unroll
        for (int q1 = 0; q1 < 4; ++q1) y[q2 + 4 * q1] = x[4 * q2 + q1];
#pragma unroll
    for (int r = 0; r < 16; ++r) x[r] = y[r];
}

// Forward DFT of 4096 points held in the padded buffer b (blockDim.x = 256);
// tw1: [15][16] = w^(m k 16), tw2: [15][256] = w^(m k), w = e^(-2 pi i / 4096)
__device__ void fft4096_r16(float2* b, const float2* __restrict__ tw1, const float2* __restrict__ tw2)
{
    const int j = threadIdx.x;
#pragma unroll 1
    for (int p = 0; p < 3; ++p) {
        const int lgNs = 4 * p, k = j & ((1 << lgNs) - 1);
        float2 x[16];
#pragma unroll
        for (int m = 0; m < 16; ++m) x[m] = b[pad16(j + 256 * m)];
        __syncthreads();
        if (p == 1) {
#pragma unroll
            for (int m = 1; m < 16; ++m) x[m] = cmul(x[m], __ldg(tw1 + (m - 1) * 16 + k));
        } else if (p == 2) {
#pragma unroll
            for (int m = 1; m < 16; ++m) x[m] = cmul(x[m], __ldg(tw2 + (m - 1) * 256 + k));
        }
        dft16(x);
        const int idxD = ((j >> lgNs) << (lgNs + 4)) + k;
#pragma unroll
        for (int r = 0; r < 16; ++r) b[pad16(idxD + (r << lgNs))] = x[r];
        __syncthreads();
    }
}

// k_filter_fft for L = 4096 in single precision (256 threads): the same
// packing, spectrum product and output as k_filter_fft, with fft4096_r16.
__global__ void __launch_bounds__(256) k_filter_fft4096(const float* __restrict__ sino, float* __restrict__ out,
                                                        const float* __restrict__ H,
                                                        const float2* __restrict__ tw16, int N, int T, int V)
{
    constexpr int L = 4096;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* b = reinterpret_cast<float2*>(smem_raw);
    const float2* tw1 = tw16;
    const float2* tw2 = tw16 + 15 * 16;
    const int g = blockIdx.y;
    size_t offa, offb;
    int stride;
    bool has_b = true;
    if (V == 4) {
        const int t = blockIdx.x >> 1, h = blockIdx.x & 1;
        offa = (((size_t)g * T + t) * N) * 4 + 2 * h;
        offb = offa + 1;
        stride = 4;
    } else {
        const int t0 = 2 * blockIdx.x;
        offa = ((size_t)g * T + t0) * N;
        offb = offa + N;
        stride = 1;
        has_b = (t0 + 1) < T;
    }
    for (int n = threadIdx.x; n < L; n += blockDim.x) {
        float2 z;
        if (V == 4) {
            z = n < N ? __ldg(reinterpret_cast<const float2*>(sino + offa + (size_t)n * 4)) : make_float2(0.f, 0.f);
        } else {
            z.x = n < N ? sino[offa + (size_t)n * stride] : 0.f;
            z.y = (n < N && has_b) ? sino[offb + (size_t)n * stride] : 0.f;
        }
        b[pad16(n)] = z;
    }
    __syncthreads();
    fft4096_r16(b, tw1, tw2);
    // W = H/L * conj(Z); y = conj(FFT(W))
    for (int m = threadIdx.x; m < L; m += blockDim.x) {
        const float2 z = b[pad16(m)];
        const float h = H[m];
        b[pad16(m)] = make_float2(h * z.x, -h * z.y);
    }
    __syncthreads();
    fft4096_r16(b, tw1, tw2);
    for (int n = threadIdx.x; n < N; n += blockDim.x) {
        const float2 v = b[pad16(n)];
        if (V == 4) {
            *reinterpret_cast<float2*>(out + offa + (size_t)n * 4) = make_float2(v.x, -v.y);
        } else {
            out[offa + (size_t)n * stride] = v.x;
            if (has_b) out[offb + (size_t)n * stride] = -v.y;
        }
    }
}

template <typename Real, int V>
void launch_filter_fft(const DevGeom<Real>& g, int G, const Real* sino, Real* out, cudaStream_t st)
{
    using C = typename Cplx<Real>::T;
    const size_t sm = 2 * (size_t)g.fft_L * sizeof(C);
    max_dynamic_smem<k_filter_fft<Real>>();
    const C* tw = reinterpret_cast<const C*>(sizeof(Real) == 4 ? (const void*)g.fft_tw : (const void*)g.fft_tw64);
    dim3 grd(V == 4 ? 2 * g.T : (g.T + 1) / 2, G);
    // 512 threads: 8 % faster than 256 at L = 4096 (more warps between the
    // stages' barriers), 1024 slower; the results do not depend on it
    // exact positions filter with the spectrum of the FP64 taps
    const Real* H = (g.exact && g.fft_h_x) ? g.fft_h_x : g.fft_h;
    if constexpr (sizeof(Real) == 4) {
        if (g.fft_L == 4096 && g.fft_tw16) {   // 3.6x the radix-4 stages at this length
            const size_t sm16 = (size_t)(4096 + 256) * sizeof(float2);
            max_dynamic_smem<k_filter_fft4096>();
            k_filter_fft4096<<<grd, 256, sm16, st>>>(sino, out, H, g.fft_tw16, g.N, g.T, V);
            return;
        }
    }
    k_filter_fft<Real><<<grd, 512, sm, st>>>(sino, out, H, tw, g.N, g.T, g.fft_L, V);
}

// Largest FFT length whose two shared-memory buffers fit in one block.
template <typename Real>
bool fft_fits(int L)
{
    return 2 * (size_t)L * 2 * sizeof(Real) <= 227 * 1024;
}

template void launch_filter_fft<float, 1>(const DevGeom<float>&, int, const float*, float*, cudaStream_t);
template void launch_filter_fft<float, 4>(const DevGeom<float>&, int, const float*, float*, cudaStream_t);
template void launch_filter_fft<double, 1>(const DevGeom<double>&, int, const double*, double*, cudaStream_t);
template bool fft_fits<float>(int);
template bool fft_fits<double>(int);

}  // namespace acu
