"""GPU parity of the projection-preprocessing path against the CPU oracle,
through the C ABI.

Bit-exact: frame averages, the 0/180 interpolation, the 27-point median and
the resample (index and comparison work, all in the reference's operation
order); the cross-correlation lag (integer, order-independent fixed-point
sums).  Tolerance: normalisation within 2 ulp-scale relative error (CUDA's
logf against the C library's); the registration's (theta, shift) within
1e-4 rad / 1e-4 of the detector width of the oracle's FP64-accumulated search,
and the recovered axis within 0.75 pixel of the synthetic offset.
"""
import numpy as np
import pytest
import torch

from acumen_gb300 import synthetic as syn
from acumen_gb300.preprocess import Preprocessor

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pp(built_lib):
    return Preprocessor()


@pytest.fixture(scope="module")
def stack(built_lib):
    ndet, nrows, nproj = 96, 12, 61
    th, raw, flats, darks = syn.projection_stack(nproj, ndet, nrows, axis_offset=-3.0, seed=11, I0=2e4)
    raw = raw.to(torch.int32).numpy().astype(np.uint16)
    flats = flats.to(torch.int32).numpy().astype(np.uint16)
    darks = darks.to(torch.int32).numpy().astype(np.uint16)
    return dict(th=th, raw=raw, flats=flats, darks=darks, ndet=ndet, nrows=nrows, nproj=nproj)


def cu(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_frame_average_bit_exact(pp, oracle, stack):
    ref = oracle.frame_average(stack["flats"].astype(np.float32))
    got = pp.frame_average(cu(stack["flats"]))          # uint16 frames
    np.testing.assert_array_equal(got.cpu().numpy(), ref)
    got = pp.frame_average(cu(stack["flats"].astype(np.float32)))
    np.testing.assert_array_equal(got.cpu().numpy(), ref)


@pytest.mark.parametrize("mode", [0, 1])
def test_normalize_matches_oracle(pp, oracle, stack, mode):
    ob = oracle.frame_average(stack["flats"].astype(np.float32))
    df = oracle.frame_average(stack["darks"].astype(np.float32))
    raw = stack["raw"][:5].astype(np.float32)
    got = pp.normalize(cu(raw), cu(ob), cu(df), mode).cpu().numpy()
    ref = np.stack([oracle.normalize(r, ob, df, mode) for r in raw])
    np.testing.assert_allclose(got, ref, rtol=5e-7, atol=5e-7)


def test_pick_angle_bit_exact(pp, oracle):
    rng = np.random.default_rng(0)
    proj = rng.standard_normal((5, 4, 6)).astype(np.float32)
    for th in (np.array([-0.7, 0.4, 90, 179.3, 180.6], np.float32), np.array([0, 45, 90, 135, 180], np.float32),
               np.array([0.3, 45, 90, 135, 179.9], np.float32)):
        for target in (0.0, 180.0):
            got = pp.pick_angle(th, cu(proj), target).cpu().numpy()
            np.testing.assert_array_equal(got, oracle.pick_angle(th, proj, target))


def test_median_and_resample_bit_exact(pp, oracle):
    rng = np.random.default_rng(1)
    a, b, c = (rng.standard_normal((10, 17)).astype(np.float32) for _ in range(3))
    np.testing.assert_array_equal(pp.median27(cu(a), cu(b), cu(c)).cpu().numpy(), oracle.median27(a, b, c))
    for theta, shift in ((0.0, 0.0), (0.013, -0.021), (-0.2, 0.05)):
        got = pp.resample(cu(b), theta, shift).cpu().numpy()
        np.testing.assert_array_equal(got, oracle.resample(b, theta, shift))


def test_median_with_nan_matches_reference_sort(pp, oracle):
    rng = np.random.default_rng(2)
    a, b, c = (rng.standard_normal((6, 7)).astype(np.float32) for _ in range(3))
    b[2, 3] = np.nan
    a[0, 0] = np.inf
    got = pp.median27(cu(a), cu(b), cu(c)).cpu().numpy()
    np.testing.assert_array_equal(got, oracle.median27(a, b, c))


def test_median_ties_zeros_and_infinities_bit_exact(pp, oracle):
    """Values from a small set (heavy ties), with signed zeros, infinities and
    a few NaN: the fast selection (no NaN, no zero among the 27) and the
    exchange sort (otherwise) both give the oracle's bits."""
    rng = np.random.default_rng(3)
    vals = np.array([1.0, 2.0, -1.5, 0.25, np.inf, -np.inf, 0.0, -0.0], np.float32)
    for frac_special in (0.0, 0.05, 0.3):
        a, b, c = (rng.choice(vals[:4], (33, 41)).astype(np.float32) for _ in range(3))
        for arr in (a, b, c):
            m = rng.random(arr.shape) < frac_special
            arr[m] = rng.choice(vals[4:], m.sum())
        b[5, 7] = np.nan
        got = pp.median27(cu(a), cu(b), cu(c)).cpu().numpy()
        ref = oracle.median27(a, b, c)
        np.testing.assert_array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_proj_to_sino_matches_oracle(pp, oracle, stack):
    ob = oracle.frame_average(stack["flats"].astype(np.float32))
    df = oracle.frame_average(stack["darks"].astype(np.float32))
    proj = np.stack([oracle.normalize(r.astype(np.float32), ob, df, 1) for r in stack["raw"]])
    got = pp.proj_to_sino(cu(proj), 0.004, -0.013).cpu().numpy()
    ref = oracle.proj_to_sino(proj, 0.004, -0.013)
    assert got.shape == (stack["nrows"], stack["nproj"], stack["ndet"] + 1)
    np.testing.assert_array_equal(got, ref)


def test_registration_matches_oracle_and_truth(pp, oracle, stack):
    ob = oracle.frame_average(stack["flats"].astype(np.float32))
    df = oracle.frame_average(stack["darks"].astype(np.float32))
    proj = np.stack([oracle.normalize(r.astype(np.float32), ob, df, 1) for r in stack["raw"]])
    p0, p180 = oracle.pick_angle(stack["th"], proj, 0.0), oracle.pick_angle(stack["th"], proj, 180.0)
    th_g, sh_g, ne_g = pp.register(cu(p0), cu(p180))
    th_o, sh_o, ne_o = oracle.register(p0, p180, red_mode=1)
    assert abs(th_g - th_o) < 1e-4 and abs(sh_g - sh_o) < 1e-4
    ndet = stack["ndet"]
    axis_true = (ndet + 2) // 2 + (-3.0)
    assert abs((ndet + 2) / 2 - sh_g * ndet - axis_true) < 0.75
    kb, ks, corr = pp.xcorr_register(cu(p0), cu(p180), 20)
    ko, kso, corr_o = oracle.xcorr_register(p0, p180, 20)
    assert kb == ko
    np.testing.assert_array_equal(corr, corr_o)
    assert ks == pytest.approx(kso, abs=1e-12)


def test_xcorr_rejects_nonfinite_input(pp):
    from acumen_gb300._lib import ACU_ERR_INVALID, AcumenError
    p0 = np.ones((4, 16), np.float32)
    p180 = np.ones((4, 16), np.float32)
    for bad in (np.nan, np.inf):
        q0 = p0.copy()
        q0[1, 7] = bad
        with pytest.raises(AcumenError, match="not finite") as ei:
            pp.xcorr_register(cu(q0), cu(p180), 3)
        assert ei.value.code == ACU_ERR_INVALID
    kb, ks, corr = pp.xcorr_register(cu(p0), cu(p180), 3)     # the context stays usable
    assert kb == 0


def test_xcorr_sums_beyond_int64(pp, oracle):
    """Sums beyond 2^63 are exact in 128 bits: the lag matches the oracle's;
    corr_out, which is int64, is refused for them."""
    from acumen_gb300._lib import ACU_ERR_UNSUPPORTED, AcumenError
    rng = np.random.default_rng(22)
    p0 = rng.uniform(30000, 40000, (40, 64)).astype(np.float32)
    p180 = (np.roll(np.ascontiguousarray(p0[:, ::-1]), 3, axis=1) * np.float32(0.9)).astype(np.float32)
    with pytest.raises(OverflowError) as ei:
        oracle.xcorr_register(p0, p180, 5)
    with pytest.raises(AcumenError) as eg:
        pp.xcorr_register(cu(p0), cu(p180), 5)
    assert eg.value.code == ACU_ERR_UNSUPPORTED
    kb, ks, corr = pp.xcorr_register(cu(p0), cu(p180), 5, want_corr=False)
    assert corr is None
    assert kb == ei.value.k_best
    assert ks == ei.value.k_sub


@pytest.mark.parametrize("reg", [0, 1])
def test_full_chain_host_buffers(pp, oracle, stack, reg):
    sino, th, sh = pp.proj_to_sino_u16(stack["raw"], stack["th"], stack["flats"], stack["darks"], norm_mode=1,
                                       reg_method=reg)
    ob = oracle.frame_average(stack["flats"].astype(np.float32))
    df = oracle.frame_average(stack["darks"].astype(np.float32))
    proj = np.stack([oracle.normalize(r.astype(np.float32), ob, df, 1) for r in stack["raw"]])
    ref = oracle.proj_to_sino(proj, th, sh)
    # normalisation differs by an ulp or so (logf); the rest is exact
    np.testing.assert_allclose(sino, ref, rtol=2e-6, atol=2e-6)
    ndet = stack["ndet"]
    axis_true = (ndet + 2) // 2 + (-3.0)
    assert abs((ndet + 2) / 2 - sh * ndet - axis_true) < 0.75


@pytest.fixture(scope="module")
def wide_stack(built_lib):
    # the config-3 detector width (2048 bins) on a few rows and projections
    ndet, nrows, nproj = 2048, 6, 25
    th, raw, flats, darks = syn.projection_stack(nproj, ndet, nrows, axis_offset=5.5, seed=5, I0=3e4)
    raw = raw.to(torch.int32).numpy().astype(np.uint16)
    flats = flats.to(torch.int32).numpy().astype(np.uint16)
    darks = darks.to(torch.int32).numpy().astype(np.uint16)
    return dict(th=th, raw=raw, flats=flats, darks=darks, ndet=ndet, nrows=nrows, nproj=nproj)


def test_chain_at_2048_bins(pp, oracle, wide_stack):
    """The preprocessing chain at the full detector width of 2048 bins (the
    odd grid 2049 after padding): median + resample + transpose bit-exact
    against the oracle on the oracle's normalised stack, the whole uint16
    chain within the normalisation's ulps, the cross-correlation lag and
    correlation vector bit-exact, and the axis within 0.75 px of the truth."""
    s = wide_stack
    ob = oracle.frame_average(s["flats"].astype(np.float32))
    df = oracle.frame_average(s["darks"].astype(np.float32))
    proj = np.stack([oracle.normalize(r.astype(np.float32), ob, df, 0) for r in s["raw"]])
    got = pp.proj_to_sino(cu(proj), 0.0021, 0.0027).cpu().numpy()
    ref = oracle.proj_to_sino(proj, 0.0021, 0.0027)
    assert got.shape == (s["nrows"], s["nproj"], s["ndet"] + 1)
    np.testing.assert_array_equal(got, ref)
    p0, p180 = oracle.pick_angle(s["th"], proj, 0.0), oracle.pick_angle(s["th"], proj, 180.0)
    kb, ks, corr = pp.xcorr_register(cu(p0), cu(p180), 64)
    ko, kso, corr_o = oracle.xcorr_register(p0, p180, 64)
    assert kb == ko
    np.testing.assert_array_equal(corr, corr_o)
    sino, th, sh = pp.proj_to_sino_u16(s["raw"], s["th"], s["flats"], s["darks"], norm_mode=0, reg_method=1)
    ref = oracle.proj_to_sino(proj, th, sh)
    np.testing.assert_allclose(sino, ref, rtol=2e-6, atol=2e-6)
    ndet = s["ndet"]
    axis_true = (ndet + 2) // 2 + 5.5
    assert abs((ndet + 2) / 2 - sh * ndet - axis_true) < 0.75
