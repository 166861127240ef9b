"""CPU pins of the oracle (tests/ only; no GPU).

The reference ships no tests or golden vectors and cannot be compiled here
(Fortran + MPI), so the restatement is pinned by known answers: closed-form
filter taps and mask values, analytic Radon transforms of ellipses, the
adjoint identity, FP32-vs-FP64 agreement, a second (numpy) restatement of the
loops in single precision, and recovery of synthetic rotation-axis offsets.
"""
import math

import numpy as np
import pytest

from acumen_gb300 import synthetic as syn


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - np.asarray(b, np.float64)) /
                 np.linalg.norm(np.asarray(b, np.float64)))


def test_filter_taps_closed_form(oracle):
    N = 33
    h = oracle.filter_taps(N, 64)
    k = np.arange(-N, N + 1)
    np.testing.assert_allclose(h, -2.0 * N / (math.pi ** 2 * (4.0 * k * k - 1)), rtol=1e-14)
    assert h[N] == pytest.approx(2 * N / math.pi ** 2)
    h32 = oracle.filter_taps(N, 32)
    np.testing.assert_allclose(h32, h, rtol=3e-7)
    np.testing.assert_array_equal(h32, h32[::-1])   # symmetric taps


def test_cmask_values(oracle):
    N, T, wpu = 65, 30, 8
    m = oracle.cmask(N, T, wpu, 64)
    c = (N - 1) // 2
    assert m[c, c] == pytest.approx(math.pi / T)
    assert m[0, 0] == 0.0 and m[-1, -1] == 0.0
    row = m[c, c:]
    assert np.all(np.diff(row) <= 1e-15)             # taper decreases outwards
    # where 0 < rtmp < 1 the value is pi*exp(1-1/(1-exp(1-1/(1-rtmp))))/T
    jx = np.arange(1, N + 1)
    X, Y = np.meshgrid(jx, jx, indexing="xy")
    r = np.sqrt((X - (N - 1) / 2 - 1) ** 2 + (Y - (N - 1) / 2 - 1) ** 2)
    rt = 1 - 2 * (r - ((N - 1) / 2 - wpu)) / wpu
    inner = (rt > 0) & (rt < 1)
    with np.errstate(all="ignore"):
        ex = math.pi * np.exp(1 - 1 / (1 - np.exp(1 - 1 / (1 - rt)))) / T
    np.testing.assert_allclose(m[inner], ex[inner], rtol=1e-12)
    # single precision: the nested exp taper amplifies rounding near its edge
    np.testing.assert_allclose(oracle.cmask(N, T, wpu, 32), m, rtol=5e-5, atol=1e-8)


def test_radon_matches_analytic_ellipses(oracle):
    N, T = 129, 60
    th = syn.angles(T)
    ell = syn.random_ellipses(7, 0.35 * N)
    img = syn.rasterize(ell, N).numpy()
    an = syn.analytic_sinogram(ell, N, th).numpy()
    r64 = oracle.radon(img, th, 64)
    assert rel(r64, an) < 0.03          # rasterisation error of the phantom
    assert rel(oracle.radon(img.astype(np.float32), th, 32), r64) < 1e-6


def test_fbp_recovers_phantom(oracle):
    N, T, wpu = 129, 120, 10
    th = syn.angles(T)
    ell = syn.random_ellipses(3, 0.35 * N)
    img = syn.rasterize(ell, N).numpy()
    an = syn.analytic_sinogram(ell, N, th).numpy()
    fbp = oracle.iradon(an, th, wpu, 64)
    inside = oracle.cmask(N, T, wpu, 64) >= math.pi / T * 0.999
    assert rel(fbp[inside], img[inside]) < 0.2
    # mean level recovered to a few percent
    assert abs(fbp[inside].mean() / img[inside].mean() - 1) < 0.05
    assert rel(oracle.iradon(an.astype(np.float32), th, wpu, 32), fbp) < 2e-6


def _numpy_filter32(x, N):
    """Second restatement of tv_hpc.F90:93-105 in float32, loop order kept."""
    h = np.empty(2 * N + 1, np.float32)
    pi = np.float32(4.0) * np.arctan(np.float32(1.0))
    for jx in range(1, 2 * N + 2):
        k = jx - 1 - N
        h[jx - 1] = -((np.float32(2.0) * np.float32(N)) / ((pi * pi) * np.float32(4 * k * k - 1)))
    out = np.empty(N, np.float32)
    for jy in range(1, N + 1):
        s = np.float32(0.0)
        for jx in range(1, N + 1):
            s = np.float32(s + np.float32(x[jx - 1] * h[jy - jx + N]))
        out[jy - 1] = s
    return out


def test_filter_f32_loop_order_bit_exact(oracle):
    N, T = 17, 3
    rng = np.random.default_rng(0)
    x = rng.standard_normal((T, N)).astype(np.float32)
    got = oracle.filter_rows(x, 32)
    for t in range(T):
        np.testing.assert_array_equal(got[t], _numpy_filter32(x[t], N))


def _numpy_backproject32(q, th, N, wpu, oracle):
    pi = np.float32(4.0) * np.arctan(np.float32(1.0))
    mid = np.float32((N + 1) // 2)
    cm = oracle.cmask(N, len(th), wpu, 32)
    out = np.zeros((N, N), np.float32)
    for jy in range(1, N + 1):
        for jx in range(1, N + 1):
            s = np.float32(0)
            for t in range(len(th)):
                ct = np.float32(np.float32(pi * np.float32(np.float32(90.0) - th[t])) / np.float32(180.0))
                yr = np.float32(np.float32(np.float32(np.sin(ct)) * np.float32(jx - mid)) +
                                np.float32(np.float32(np.cos(ct)) * np.float32(jy - mid)))
                yr = np.float32(yr + mid)
                y1 = int(np.floor(yr))
                if y1 > 1 and y1 + 1 < N + 1:
                    s = np.float32(s + np.float32(q[t, y1 - 1] * np.float32(np.float32(y1 + 1) - yr)))
                    s = np.float32(s + np.float32(q[t, y1] * np.float32(yr - np.float32(y1))))
            out[jy - 1, jx - 1] = np.float32(cm[jy - 1, jx - 1] * s)
    return out


def test_backproject_f32_second_restatement(oracle):
    N, T, wpu = 15, 7, 2
    th = syn.angles(T)
    rng = np.random.default_rng(1)
    q = rng.standard_normal((T, N)).astype(np.float32)
    got = oracle.backproject(q, th, wpu, 32)
    ref = _numpy_backproject32(q, th, N, wpu, oracle)
    # numpy's float32 sin/cos may differ from libm sinf/cosf by an ulp
    np.testing.assert_allclose(got, ref, rtol=2e-5, atol=2e-6)


def test_radon_adjoint_identity(oracle):
    N, T = 33, 20
    th = syn.angles(T)
    rng = np.random.default_rng(2)
    x = rng.standard_normal((N, N))
    y = rng.standard_normal((T, N))
    lhs = np.vdot(oracle.radon(x, th, 64), y)
    rhs = np.vdot(x, oracle.radon_adjoint(y, th, 64))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


def test_tvopt_no_iterations_is_fbp(oracle):
    N, T, wpu = 33, 24, 4
    th = syn.angles(T)
    ell = syn.random_ellipses(5, 0.3 * N)
    f = syn.analytic_sinogram(ell, N, th).numpy()
    tv, fbp = oracle.tvopt(f, th, wpu, 1, 0, 5, 0.05, 1.0, prec=64)
    np.testing.assert_array_equal(tv, fbp)
    np.testing.assert_allclose(fbp, oracle.iradon(f, th, wpu, 64), rtol=0, atol=0)


def test_tvopt_f32_tracks_f64(oracle):
    N, T, wpu = 65, 45, 6
    th = syn.angles(T)
    ell = syn.random_ellipses(11, 0.3 * N)
    f = syn.analytic_sinogram(ell, N, th).numpy()
    tv64, _ = oracle.tvopt(f, th, wpu, 1, 5, 5, 0.05, 1.0, prec=64)
    tv32, _ = oracle.tvopt(f.astype(np.float32), th, wpu, 1, 5, 5, 0.05, 1.0, prec=32, red_mode=1)
    inside = oracle.cmask(N, T, wpu, 64) > 0
    assert rel(tv32[inside], tv64[inside]) < 1e-4


def test_median27_matches_numpy(oracle):
    rng = np.random.default_rng(3)
    a, b, c = (rng.standard_normal((9, 13)).astype(np.float32) for _ in range(3))
    got = oracle.median27(a, b, c)
    stack = []
    for img in (a, b, c):
        p = np.pad(img, 1, mode="edge")
        for dy in range(3):
            for dx in range(3):
                stack.append(p[dy:dy + 9, dx:dx + 13])
    np.testing.assert_array_equal(got, np.median(np.stack(stack), axis=0).astype(np.float32))


def test_normalize_modes(oracle):
    rng = np.random.default_rng(4)
    I = rng.uniform(50, 5000, (8, 8)).astype(np.float32)
    ob = rng.uniform(0.5, 6000, (8, 8)).astype(np.float32)
    df = rng.uniform(0, 200, (8, 8)).astype(np.float32)
    m0 = oracle.normalize(I, ob, df, 0)
    np.testing.assert_allclose(m0, -np.log(I / np.maximum(ob, 1.0)), rtol=1e-6, atol=1e-6)
    m1 = oracle.normalize(I, ob, df, 1)
    ex = -np.log(np.maximum(I - df, 1e-16) / np.maximum(ob - df, 1.0))
    np.testing.assert_allclose(m1, ex, rtol=1e-5, atol=1e-5)


def test_pick_angle_exact_and_interpolated(oracle):
    proj = np.stack([np.full((2, 3), v, np.float32) for v in (10.0, 20.0, 30.0, 40.0)])
    th = np.array([-1.0, 1.0, 179.0, 181.0], np.float32)
    assert oracle.minloc_abs(th, 0.0) == 1
    np.testing.assert_allclose(oracle.pick_angle(th, proj, 0.0), 15.0)       # between -1 and 1
    np.testing.assert_allclose(oracle.pick_angle(th, proj, 180.0), 35.0)
    th2 = np.array([0.0, 90.0, 180.0, 200.0], np.float32)
    np.testing.assert_array_equal(oracle.pick_angle(th2, proj, 0.0), proj[0])
    np.testing.assert_array_equal(oracle.pick_angle(th2, proj, 180.0), proj[2])


def _pair_with_offset(ndet, nrows, offset, seed):
    th, raw, flats, darks = syn.projection_stack(181, ndet, nrows, offset, seed, I0=1e5)
    raw = raw.to(__import__("torch").int32).numpy().astype(np.float32)
    ob = flats.to(__import__("torch").int32).numpy().astype(np.float32).mean(0)
    df = darks.to(__import__("torch").int32).numpy().astype(np.float32).mean(0)
    p = -np.log(np.maximum(raw - df, 1e-16) / np.maximum(ob - df, 1.0))
    return th, p


@pytest.mark.parametrize("offset", [-5.0, 3.0])
def test_register_recovers_axis_offset(oracle, offset):
    ndet, nrows = 64, 8
    th, p = _pair_with_offset(ndet, nrows, offset, seed=5)
    p0, p180 = p[0], p[-1]
    theta, shift, ne = oracle.register(p0, p180, red_mode=1)
    add = 1 if ndet % 2 == 0 else 0
    # the synthetic axis sits at 1-based detector coordinate (ndet+add+1)//2 + offset
    axis_true = (ndet + add + 1) // 2 + offset
    # resample moves the source axis to the mirror centre (ndet+add+1)/2
    axis_src = (ndet + add + 1) / 2 - shift * ndet
    assert abs(axis_src - axis_true) < 0.75
    assert abs(theta) < 0.01
    k, ksub, corr = oracle.xcorr_register(p0, p180, 24)
    # xcorr lag k puts the 0-based axis at (ndet - 1 + k) / 2
    k_true = 2 * (axis_true - 1) - (ndet - 1)
    assert abs(k - k_true) <= 1
    assert abs(ksub - k_true) < 0.5


def _xcorr_exact(p0, p180, kmax):
    """The correlation sums with Python integers: floor(p0*p180*2^32) summed
    without bound (float64 products of two float32 values are exact)."""
    nrows, ndet = p0.shape
    a, b = p0.astype(np.float64), p180.astype(np.float64)
    out = []
    for k in range(-kmax, kmax + 1):
        s = 0
        for x in range(ndet):
            xm = ndet - 1 - x + k
            if 0 <= xm < ndet:
                s += sum(int(np.floor(v)) for v in a[:, x] * b[:, xm] * 4294967296.0)
        out.append(s)
    return out


def test_xcorr_sums_are_exact_integers(oracle):
    rng = np.random.default_rng(21)
    p0 = rng.uniform(-3, 3, (5, 23)).astype(np.float32)
    p180 = rng.uniform(-3, 3, (5, 23)).astype(np.float32)
    k, ksub, corr = oracle.xcorr_register(p0, p180, 6)
    ref = _xcorr_exact(p0, p180, 6)
    assert corr.tolist() == ref
    assert k == int(np.argmax(ref)) - 6


def test_xcorr_rejects_nonfinite_and_out_of_range_products(oracle):
    p0 = np.ones((4, 16), np.float32)
    p180 = np.ones((4, 16), np.float32)
    for bad in (np.nan, np.inf, 5e4):          # 5e4 * 1 is fine alone; 5e4^2 >= 2^31
        q0, q180 = p0.copy(), p180.copy()
        q0[2, 5] = bad
        q180[2, 16 - 1 - 5] = bad if bad == 5e4 else 1.0
        with pytest.raises(ValueError):
            oracle.xcorr_register(q0, q180, 3)


def test_xcorr_sums_beyond_int64_keep_the_exact_argmax(oracle):
    # products ~1.2e9 (below 2^31) over 40 x 64 pixels: sums ~1.3e22 > 2^63
    rng = np.random.default_rng(22)
    p0 = rng.uniform(30000, 40000, (40, 64)).astype(np.float32)
    p180 = np.ascontiguousarray(p0[:, ::-1])
    p180 = np.roll(p180, 3, axis=1) * np.float32(0.9)
    with pytest.raises(OverflowError) as ei:
        oracle.xcorr_register(p0, p180, 5)
    ref = _xcorr_exact(p0, p180, 5)
    assert max(abs(v) for v in ref) > 2 ** 63
    assert ei.value.k_best == int(np.argmax(ref)) - 5
