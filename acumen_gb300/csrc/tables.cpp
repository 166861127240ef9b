// Host-side geometry tables of one reconstruction grid (int_radon,
// tomography/tv_hpc.F90:11-78) in single or double precision.
//
// Built with -ffp-contract=off so that single precision is evaluated in the
// reference's operation order with the C library's sinf/cosf/expf/sqrtf; the
// tables are uploaded once and every kernel reads them, so the mask, the
// filter taps and the per-angle sines are identical to the reference's.
#include "tables.h"

#include <cmath>
#include <complex>

namespace acu {

template <typename Real>
static Real r_atan(Real x) { return std::atan(x); }
template <typename Real>
static Real r_sin(Real x) { return std::sin(x); }
template <typename Real>
static Real r_cos(Real x) { return std::cos(x); }
template <typename Real>
static Real r_exp(Real x) { return std::exp(x); }
template <typename Real>
static Real r_sqrt(Real x) { return std::sqrt(x); }

template <typename Real>
void make_tables(int N, int T, const float* theta, int wpu, HostTables<Real>& out)
{
    const Real pi = Real(4) * r_atan<Real>(Real(1));
    out.N = N;
    out.T = T;
    out.mid = (Real)((N + 1) / 2);
    // filter taps, tv_hpc.F90:53-56
    out.filt.resize(2 * (size_t)N + 1);
    for (int jx = 1; jx <= 2 * N + 1; ++jx) {
        long k = (long)(jx - 1 - N);
        long den = 4 * k * k - 1;
        out.filt[jx - 1] = -((Real(2) * (Real)N) / ((pi * pi) * (Real)den));
    }
    // mask, tv_hpc.F90:58-74
    out.cmask.resize((size_t)N * N);
    const Real rad_n = (Real)(N - 1) / Real(2) - (Real)wpu;
    for (int jy = 1; jy <= N; ++jy) {
        for (int jx = 1; jx <= N; ++jx) {
            Real ax = ((Real)jx - ((Real)N - Real(1)) / Real(2)) - Real(1);
            Real ay = ((Real)jy - ((Real)N - Real(1)) / Real(2)) - Real(1);
            Real rr = r_sqrt<Real>(ax * ax + ay * ay);
            Real rtmp = Real(1) - (Real(2) * (rr - rad_n)) / (Real)wpu;
            Real v;
            if (rtmp <= Real(0)) {
                v = Real(0);
            } else if (rtmp >= Real(1)) {
                v = pi / (Real)T;
            } else {
                Real in = r_exp<Real>(Real(1) - Real(1) / (Real(1) - rtmp));
                v = (pi * r_exp<Real>(Real(1) - Real(1) / (Real(1) - in))) / (Real)T;
            }
            out.cmask[(size_t)(jy - 1) * N + (jx - 1)] = v;
        }
    }
    // angle tables, tv_hpc.F90:113 and :142
    out.sc_bp.resize(2 * (size_t)T);
    out.sc_fp.resize(2 * (size_t)T);
    for (int t = 0; t < T; ++t) {
        Real th = (Real)theta[t];
        Real ctb = (pi * (Real(90) - th)) / Real(180);
        Real ctf = (pi * (th - Real(90))) / Real(180);
        out.sc_bp[2 * t] = r_sin<Real>(ctb);
        out.sc_bp[2 * t + 1] = r_cos<Real>(ctb);
        out.sc_fp[2 * t] = r_sin<Real>(ctf);
        out.sc_fp[2 * t + 1] = r_cos<Real>(ctf);
    }
    // exact-position split (single-precision kernels, option 8): k = bits of
    // mid bounds every pixel offset, q = 23 - k keeps s_a * offset and
    // c_a * offset + mid within 24 significant bits
    {
        int k = 0;
        while ((1L << k) <= (long)((N + 1) / 2)) ++k;
        out.xq = 23 - k;
        const double pid = 4.0 * std::atan(1.0);
        out.xsc_bp.resize(4 * (size_t)T);
        out.xsc_fp.resize(4 * (size_t)T);
        // A sine or cosine below 1e-12 is the FP64 rounding residue of a
        // grid-aligned angle (cos(pi/2) evaluates to 6.1e-17): its true value
        // is 0.  Kept, it would move samples that lie exactly on a cell edge
        // by ~1e-15 px to the other side of the edge, where the FP64
        // evaluation rounds them back onto it; at the grid border that flips
        // the validity test (tv_hpc.F90:117,149) against FP64.
        auto split = [&](double v, float& a, float& r) {
            if (std::fabs(v) < 1e-12) v = 0.0;
            const double av = std::ldexp(std::nearbyint(std::ldexp(v, out.xq)), -out.xq);
            a = (float)av;
            r = (float)(v - av);
        };
        for (int t = 0; t < T; ++t) {
            const double th = (double)theta[t];
            const double ctb = (pid * (90.0 - th)) / 180.0, ctf = (pid * (th - 90.0)) / 180.0;
            split(std::sin(ctb), out.xsc_bp[4 * t], out.xsc_bp[4 * t + 2]);
            split(std::cos(ctb), out.xsc_bp[4 * t + 1], out.xsc_bp[4 * t + 3]);
            split(std::sin(ctf), out.xsc_fp[4 * t], out.xsc_fp[4 * t + 2]);
            split(std::cos(ctf), out.xsc_fp[4 * t + 1], out.xsc_fp[4 * t + 3]);
        }
    }
    // FFT form of the same filter: circular kernel of length L >= 2N-2 holding
    // taps -(N-1)..(N-1) (the two taps +-(N-1) are equal and share one slot
    // when L = 2N-2); its DFT is real because the kernel is symmetric.
    int L = 1, lg = 0;
    while (L < 2 * N - 2) { L <<= 1; ++lg; }
    if (L < 16) { L = 16; lg = 4; }
    out.fft_L = L;
    out.fft_log2L = lg;
    const double pid = 4.0 * std::atan(1.0);
    // fft_h = DFT(c) / L (the inverse transform's 1/L folded in), in double:
    // an iterative radix-2 transform (L is a power of two) with every twiddle
    // from cos/sin of its own angle; the spectrum of the symmetric kernel is
    // real, so the (round-off) imaginary part is dropped
    auto spectrum = [&](const std::vector<double>& c, std::vector<Real>& h) {
        std::vector<std::complex<double>> a(L);
        for (int k = 0; k < L; ++k) a[k] = c[k];
        for (int i = 1, j = 0; i < L; ++i) {   // bit reversal
            int bit = L >> 1;
            for (; j & bit; bit >>= 1) j ^= bit;
            j ^= bit;
            if (i < j) std::swap(a[i], a[j]);
        }
        std::vector<std::complex<double>> w(L / 2);
        for (int k = 0; k < L / 2; ++k) w[k] = std::polar(1.0, -2.0 * pid * (double)k / (double)L);
        for (int len = 2; len <= L; len <<= 1) {
            const int step = L / len;
            for (int i = 0; i < L; i += len)
                for (int k = 0; k < len / 2; ++k) {
                    const std::complex<double> u = a[i + k], v = a[i + k + len / 2] * w[k * step];
                    a[i + k] = u + v;
                    a[i + k + len / 2] = u - v;
                }
        }
        h.resize(L);
        for (int m = 0; m < L; ++m) h[m] = (Real)(a[m].real() / (double)L);
    };
    std::vector<double> c(L, 0.0), cx(L, 0.0);
    for (int k = -(N - 1); k <= N - 1; ++k) {
        c[((k % L) + L) % L] = (double)out.filt[k + N];
        // the same tap in FP64: the ramp kernel sums to almost nothing, so the
        // single-precision taps' rounding alone moves a filtered row by ~1e-5
        // of its norm at N = 2049; exact positions filter with these instead
        cx[((k % L) + L) % L] = -(2.0 * (double)N) / ((pid * pid) * (double)(4L * k * k - 1));
    }
    spectrum(c, out.fft_h);
    spectrum(cx, out.fft_h_x);
    out.fft_tw.resize(2 * (size_t)L);   // (cos, sin) of -2 pi k / L, k < L
    for (int k = 0; k < L; ++k) {
        double a = -2.0 * pid * (double)k / (double)L;
        out.fft_tw[2 * k] = std::cos(a);
        out.fft_tw[2 * k + 1] = std::sin(a);
    }
    out.fft_tw16.clear();
    if (L == 4096) {
        auto put = [&](long e) {
            const double a = -2.0 * pid * (double)(e % L) / (double)L;
            out.fft_tw16.push_back(std::cos(a));
            out.fft_tw16.push_back(std::sin(a));
        };
        for (int m = 1; m < 16; ++m)
            for (int k = 0; k < 16; ++k) put((long)m * k * 16);
        for (int m = 1; m < 16; ++m)
            for (int k = 0; k < 256; ++k) put((long)m * k);
    }
}

template void make_tables<float>(int, int, const float*, int, HostTables<float>&);
template void make_tables<double>(int, int, const float*, int, HostTables<double>&);

}  // namespace acu
