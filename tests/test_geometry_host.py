"""Host-side checks of two geometric facts the single-precision kernels rely
on, by emulating their float32 arithmetic in numpy (no GPU):

* exact sample positions (ACU_OPT_POSITIONS = 1, csrc/common.cuh exact_coord,
  tables in csrc/tables.cpp): each FP64 sine/cosine is split into a multiple of
  2^-q (q = 23 - bits of m) and a float32 remainder; the high part of
  a*k1 + b*k2 + m is then exact in float32, and the cell and fraction agree
  with FP64 to ~1e-7 px;
* the projector's step clipping (csrc/common.cuh valid_steps): the steps
  it keeps, with a two-step margin, contain every sample of the ray that
  passes the reference's validity test (tomography/tv_hpc.F90:149).
"""
import numpy as np
import pytest

from acumen_gb300 import synthetic as syn

f32 = np.float32


def fma32(a, b, c):
    """float32 fused multiply-add: the float64 product of two float32 values is
    exact, so one rounding of product + c to float32 (done in float64 first,
    which for these magnitudes does not double-round)."""
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def split(v, q):
    if abs(v) < 1e-12:          # the FP64 residue of a grid-aligned angle (csrc/tables.cpp)
        v = 0.0
    a = np.ldexp(np.rint(np.ldexp(v, q)), -q)
    return f32(a), f32(v - a)


def exact_coord(a_hi, b_hi, a_lo, b_lo, k1, k2, mid):
    hi = fma32(a_hi, k1, fma32(b_hi, k2, mid))
    lo = fma32(a_lo, k1, f32(b_lo * k2))
    fl = np.floor(hi)
    fr = f32(f32(hi - fl) + lo)
    f2 = np.floor(fr)
    return float(fl) + float(f2), float(f32(fr - f2))


@pytest.mark.parametrize("N", [725, 2049, 2897, 4095])
def test_exact_positions_match_fp64(N):
    mid = (N + 1) // 2
    k = 0
    while (1 << k) <= mid:
        k += 1
    q = 23 - k
    rng = np.random.default_rng(N)
    worst = 0.0
    for th in rng.uniform(0, 180, 24).astype(np.float32):
        ct = np.pi * (90.0 - float(th)) / 180.0            # backprojection convention
        sv, cv = np.sin(ct), np.cos(ct)
        sa, sr = split(sv, q)
        ca, cr = split(cv, q)
        for x, y in rng.integers(1, N + 1, size=(300, 2)):
            dx, dy = f32(x - mid), f32(y - mid)
            hi = fma32(sa, dx, fma32(ca, dy, f32(mid)))
            exact_hi = float(sa) * float(dx) + float(ca) * float(dy) + mid
            if abs(exact_hi) < 2 ** (k + 1):
                assert float(hi) == exact_hi                # the high part is exact
            cell, frac = exact_coord(sa, ca, sr, cr, dx, dy, f32(mid))
            v = sv * (x - mid) + cv * (y - mid) + mid
            if 1 < v < N:
                assert cell == np.floor(v) or abs(v - round(v)) < 1e-6
                worst = max(worst, abs(cell + frac - v))
    assert worst < 1.5e-7, worst


def valid_steps(s, c, dy, mid, N):
    """float32 restatement of valid_steps (csrc/common.cuh)."""
    a, b = f32(-1e30), f32(1e30)

    def axis(slope, off, a, b):
        if abs(slope) < f32(1e-3):
            return a, b
        t0 = (f32(2) - off) / slope
        t1 = (f32(N) - off) / slope
        return max(a, min(t0, t1)), min(b, max(t0, t1))

    a, b = axis(c, f32(mid - s * dy), a, b)
    a, b = axis(s, f32(mid + c * dy), a, b)
    lo = max(1, int(np.floor(max(a + mid, f32(-1e8)))) - 2)
    hi = min(N, int(np.ceil(min(b + mid, f32(1e8)))) + 2)
    return lo, hi


@pytest.mark.parametrize("N", [64, 129, 513])
def test_step_clipping_keeps_every_valid_sample(N):
    mid = f32((N + 1) // 2)
    ths = np.concatenate([syn.angles(37), [90.0, 0.0, 45.0, 135.0, 89.9999, 1e-5, 44.99999]]).astype(np.float32)
    pi = f32(4) * np.arctan(f32(1))
    jx = np.arange(1, N + 1, dtype=np.float32)
    dxv = jx - mid
    for th in ths:
        ct = (pi * (th - f32(90))) / f32(180)                 # projector convention, float32
        s, c = f32(np.sin(ct)), f32(np.cos(ct))
        for jy in range(1, N + 1, max(1, N // 48)):
            dy = f32(jy) - mid
            lo, hi = valid_steps(s, c, dy, mid, N)
            xr = (c * dxv - s * dy) + mid
            yr = (s * dxv + c * dy) + mid
            x1, y1 = np.floor(xr).astype(int), np.floor(yr).astype(int)
            ok = (np.minimum(x1, y1) > 1) & (np.maximum(x1, y1) < N)
            idx = np.nonzero(ok)[0] + 1
            if idx.size:
                assert lo <= idx.min() and idx.max() <= hi, (th, jy, lo, hi, idx.min(), idx.max())


def band_steps(s, c, dy, mid, N, ylo, yhi, lo, hi):
    """float32 restatement of band_steps (csrc/kernels_lines.cu)."""
    off = f32(mid + f32(c * dy))
    y0, y1 = f32(ylo - 1), f32(yhi + 2)
    if abs(s) < f32(1e-3):
        climb = f32(abs(s) * f32(N)) + f32(2)
        if off + climb < y0 or off - climb > y1:
            return 1, 0
        return lo, hi
    t0, t1 = (y0 - off) / s, (y1 - off) / s
    return max(lo, int(np.floor(f32(min(t0, t1) + mid))) - 2), min(hi, int(np.ceil(f32(max(t0, t1) + mid))) + 2)


@pytest.mark.parametrize("N, H", [(64, 7), (129, 16), (300, 41)])
def test_band_walk_visits_every_sample_once_in_step_order(N, H):
    """Projector variant 6 walks the cell rows 2..N-1 in bands of H rows: each
    valid sample of a ray lies in the step range that band_steps keeps for
    exactly the band of its cell row, and the bands in launch order (upward
    for sin >= 0, downward otherwise) meet a ray's samples in step order."""
    mid = f32((N + 1) // 2)
    nb = max(1, (N - 2 + H - 1) // H)
    ths = np.concatenate([syn.angles(29), [90.0, 0.0, 45.0, 135.0, 89.9999, 90.0001, 1e-5, 179.99]]).astype(np.float32)
    pi = f32(4) * np.arctan(f32(1))
    jx = np.arange(1, N + 1, dtype=np.float32)
    dxv = jx - mid
    for th in ths:
        ct = (pi * (th - f32(90))) / f32(180)
        s, c = f32(np.sin(ct)), f32(np.cos(ct))
        for jy in range(1, N + 1, max(1, N // 40)):
            dy = f32(jy) - mid
            lo, hi = valid_steps(s, c, dy, mid, N)
            xr = (c * dxv - s * dy) + mid
            yr = (s * dxv + c * dy) + mid
            x1, y1 = np.floor(xr).astype(int), np.floor(yr).astype(int)
            ok = (np.minimum(x1, y1) > 1) & (np.maximum(x1, y1) < N)
            seen = []
            for k in range(nb):
                b = k if s >= 0 else nb - 1 - k
                ylo, yhi = 2 + b * H, min(N - 1, 1 + (b + 1) * H)
                blo, bhi = band_steps(s, c, dy, mid, N, ylo, yhi, lo, hi)
                inband = ok & (y1 >= ylo) & (y1 <= yhi)
                idx = np.nonzero(inband)[0] + 1
                if idx.size:
                    assert blo <= idx.min() and idx.max() <= bhi, (th, jy, b, blo, bhi, idx.min(), idx.max())
                seen.extend(idx.tolist())
            assert seen == (np.nonzero(ok)[0] + 1).tolist(), (th, jy)


@pytest.mark.parametrize("N", [25, 49, 725])
def test_grid_aligned_angles_keep_fp64_validity(N):
    """At 0, 90 and 180 degrees one of the FP64 sines/cosines is a rounding
    residue (6.1e-17 instead of 0).  Samples then sit exactly on cell edges;
    FP64 rounds the residue's product away at the grid border, so the exact
    tables hold 0 there.  Every projector sample (tv_hpc.F90:144-149, with
    detector offsets too) then passes or fails the validity test exactly as in
    FP64, and valid samples fall in the same cell wherever the FP64 fraction
    is not on an edge."""
    mid = (N + 1) // 2
    k = 0
    while (1 << k) <= mid:
        k += 1
    q = 23 - k
    for th in (0.0, 90.0, 180.0):
        ct = np.pi * (float(np.float32(th)) - 90.0) / 180.0        # projector convention
        sv, cv = np.sin(ct), np.cos(ct)
        sa, sr = split(sv, q)
        ca, cr = split(cv, q)
        # every sample near the grid border (where validity is decided) and
        # a sparse set of interior samples
        near = [j for j in range(1, N + 1) if j <= 4 or j >= N - 3 or j % 97 == 0]
        for o in (0.0, -1.3, 0.7):
            for jy in range(1, N + 1):
                dy = f32(jy - mid)
                for jx in (range(1, N + 1) if jy in near else near):
                    dx = f32(jx - mid)
                    # exact mode with a detector offset o (ProjRay<float, true>)
                    bxl = fma32(-sa, f32(o), fma32(-sr, f32(o), f32(-sr * dy)))
                    byl = fma32(ca, f32(o), fma32(cr, f32(o), f32(cr * dy)))
                    cx, fx = exact_coord(ca, -sa, cr, -sr, dx, dy, f32(mid)) if o == 0 else \
                        _split_floor(fma32(ca, dx, fma32(-sa, dy, f32(mid))), fma32(cr, dx, bxl))
                    cy, fy = exact_coord(sa, ca, sr, cr, dx, dy, f32(mid)) if o == 0 else \
                        _split_floor(fma32(sa, dx, fma32(ca, dy, f32(mid))), fma32(sr, dx, byl))
                    # FP64 in the oracle's operation order
                    xr = (cv * (jx - mid) - sv * (jy + o - mid)) + mid
                    yr = (sv * (jx - mid) + cv * (jy + o - mid)) + mid
                    x1, y1 = int(np.floor(xr)), int(np.floor(yr))
                    ok64 = min(x1, y1) > 1 and max(x1, y1) + 1 < N + 1
                    ok32 = min(cx, cy) > 1 and max(cx, cy) + 1 < N + 1
                    assert ok32 == ok64, (th, o, jx, jy, xr, yr, cx, cy)
                    if ok64 and 1e-9 < xr - x1 < 1 - 1e-9:
                        assert cx == x1
                    if ok64 and 1e-9 < yr - y1 < 1 - 1e-9:
                        assert cy == y1


def _split_floor(hi, lo):
    fl = np.floor(hi)
    fr = f32(f32(hi - fl) + lo)
    f2 = np.floor(fr)
    return float(fl) + float(f2), float(f32(fr - f2))
