// Host geometry tables (see tables.cpp).
#pragma once
#include <vector>

namespace acu {

template <typename Real>
struct HostTables {
    int N = 0, T = 0;
    Real mid = 0;
    std::vector<Real> filt;    // 2N+1
    std::vector<Real> cmask;   // N*N
    std::vector<Real> sc_bp;   // 2T
    std::vector<Real> sc_fp;   // 2T
    // Exact-position split of the FP64 sines and cosines (both conventions):
    // [T][4] = (s_a, c_a, s_r, c_r) with s_a a multiple of 2^-xq, so that
    // s_a * k is exact in single precision for every pixel offset |k| <= mid,
    // and s_r = s - s_a rounded to single precision.
    std::vector<float> xsc_bp, xsc_fp;
    int xq = 0;
    std::vector<Real> fft_h;   // L: spectrum of the taps above (the reference's arithmetic)
    std::vector<Real> fft_h_x; // L: spectrum of the taps evaluated in FP64 (exact positions)
    std::vector<double> fft_tw;  // 2*L: cos, sin of -2 pi k / L
    // L = 4096 only: the radix-16 passes' twiddles w^(m k 16) [15][16] then
    // w^(m k) [15][256], m = 1..15, as (cos, sin) pairs (w = e^(-2 pi i / L))
    std::vector<double> fft_tw16;
    int fft_L = 0, fft_log2L = 0;
};

template <typename Real>
void make_tables(int N, int T, const float* theta, int wpu, HostTables<Real>& out);

}  // namespace acu
