"""GPU parity of the Radon operators against the CPU oracle, through the C ABI.

Tolerances (relative L2): single precision vs the oracle's single-precision
restatement 1e-5 (FBP bar) and vs its FP64 restatement 1e-5; the double
precision kernels vs the FP64 oracle 1e-11.  The adjoint pair passes the
dot-product test to single-precision round-off (1e-5) and to 1e-12 in FP64.
"""
import numpy as np
import pytest
import torch

from acumen_gb300 import synthetic as syn
from acumen_gb300.tomography import Tomography

pytestmark = pytest.mark.gpu

FBP_TOL = 1e-5


def rel(a, b):
    a = np.asarray(a.cpu() if isinstance(a, torch.Tensor) else a, np.float64)
    b = np.asarray(b.cpu() if isinstance(b, torch.Tensor) else b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def case(built_lib, oracle):
    N, T, wpu = 129, 90, 10
    th = syn.angles(T)
    ells = [syn.random_ellipses(s, 0.35 * N) for s in range(6)]
    img = np.stack([syn.rasterize(e, N).numpy() for e in ells])
    sino = np.stack([syn.analytic_sinogram(e, N, th).numpy() for e in ells])
    return dict(N=N, T=T, wpu=wpu, th=th, img=img, sino=sino)


@pytest.mark.parametrize("S", [1, 6])
@pytest.mark.parametrize("filt", [0, 1])
def test_iradon_matches_oracle(case, oracle, S, filt):
    t = Tomography(case["N"], case["th"], case["wpu"])
    t.set_option(1, filt)
    sino = case["sino"][:S].astype(np.float32)
    got = t.iradon(torch.from_numpy(sino).cuda())
    ref32 = oracle.iradon(sino, case["th"], case["wpu"], 32)
    ref64 = oracle.iradon(sino.astype(np.float64), case["th"], case["wpu"], 64)
    assert rel(got, ref32) < FBP_TOL
    assert rel(got, ref64) < FBP_TOL
    # host-buffer entry point gives the same numbers
    host = t.iradon(sino)
    np.testing.assert_array_equal(host, got.cpu().numpy())


@pytest.mark.parametrize("S", [1, 6])
def test_radon_matches_oracle(case, oracle, S):
    t = Tomography(case["N"], case["th"], case["wpu"])
    img = case["img"][:S].astype(np.float32)
    got = t.radon(torch.from_numpy(img).cuda())
    ref32 = oracle.radon(img, case["th"], 32)
    ref64 = oracle.radon(img.astype(np.float64), case["th"], 64)
    assert rel(got, ref32) < 1e-6
    assert rel(got, ref64) < 1e-6


def test_radon_random_image_full_support(case, oracle):
    """Random values reach the image border, where the validity test
    (tv_hpc.F90:149) decides.  At grid-aligned angles the reference's single
    precision cos(-pi/2) = -4.4e-8 moves samples of the border bins just below
    x = 2 and drops them, where double precision keeps them: the kernels follow
    the single-precision geometry, so they match the FP32 restatement tightly
    and the FP64 one only away from the border."""
    rng = np.random.default_rng(0)
    N = case["N"]
    x = rng.standard_normal((5, N, N)).astype(np.float32)
    t = Tomography(N, case["th"], case["wpu"])
    t.set_option(8, 0)                     # the reference's single-precision positions
    got = t.radon(torch.from_numpy(x).cuda())
    assert rel(got, oracle.radon(x, case["th"], 32)) < 1e-6
    inner = x.copy()
    inner[:, :3, :] = inner[:, -3:, :] = inner[:, :, :3] = inner[:, :, -3:] = 0
    got = t.radon(torch.from_numpy(inner).cuda())
    assert rel(got, oracle.radon(inner.astype(np.float64), case["th"], 64)) < 1e-5


def test_filter_and_backproject_halves(case, oracle):
    t = Tomography(case["N"], case["th"], case["wpu"])
    sino = torch.from_numpy(case["sino"][:4].astype(np.float32)).cuda()
    q_fft = t.filter(sino)
    t.set_option(1, 1)
    q_dir = t.filter(sino)
    ref = oracle.filter_rows(case["sino"][:4], 64)
    assert rel(q_dir, ref) < 1e-6
    assert rel(q_fft, ref) < 1e-5
    img = t.backproject(q_dir)
    assert rel(img, oracle.backproject(q_dir.cpu().numpy().astype(np.float64), case["th"], case["wpu"], 64)) < 1e-6
    # double precision halves against the FP64 oracle
    s64 = sino.double()
    for filt in (0, 1):
        t.set_option(1, filt)
        q64 = t.filter(s64)
        assert q64.dtype == torch.float64 and rel(q64, oracle.filter_rows(s64.cpu().numpy(), 64)) < 1e-11
    img64 = t.backproject(q64)
    assert rel(img64, oracle.backproject(q64.cpu().numpy(), case["th"], case["wpu"], 64)) < 1e-11
    with pytest.raises(TypeError):
        t.backproject(q64.cpu().numpy())


@pytest.mark.parametrize("S", [1, 4])
def test_adjoint_dot_product_f32(case, S):
    rng = np.random.default_rng(1)
    N, T = case["N"], case["T"]
    x = torch.from_numpy(rng.standard_normal((S, N, N)).astype(np.float32)).cuda()
    y = torch.from_numpy(rng.standard_normal((S, T, N)).astype(np.float32)).cuda()
    t = Tomography(N, case["th"], case["wpu"])
    lhs = torch.sum(t.radon(x).double() * y.double()).item()
    rhs = torch.sum(x.double() * t.radon_adjoint(y).double()).item()
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)


def test_adjoint_matches_oracle_and_f64_identity(case, oracle):
    rng = np.random.default_rng(2)
    N, T = case["N"], case["T"]
    y = rng.standard_normal((T, N))
    x = rng.standard_normal((N, N))
    t = Tomography(N, case["th"], case["wpu"])
    adj64 = t.radon_adjoint(torch.from_numpy(y).cuda())
    assert rel(adj64, oracle.radon_adjoint(y, case["th"], 64)) < 1e-11
    lhs = float(np.vdot(t.radon(torch.from_numpy(x).cuda()).cpu().numpy(), y))
    rhs = float(np.vdot(x, adj64.cpu().numpy()))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


def test_f64_kernels_match_f64_oracle(case, oracle):
    t = Tomography(case["N"], case["th"], case["wpu"])
    img = torch.from_numpy(case["img"][:2]).cuda()
    sino = torch.from_numpy(case["sino"][:2]).cuda()
    assert rel(t.radon(img), oracle.radon(case["img"][:2], case["th"], 64)) < 1e-11
    t.set_option(1, 1)
    assert rel(t.iradon(sino), oracle.iradon(case["sino"][:2], case["th"], case["wpu"], 64)) < 1e-11
    t.set_option(1, 0)
    assert rel(t.iradon(sino), oracle.iradon(case["sino"][:2], case["th"], case["wpu"], 64)) < 1e-11


def test_even_grid_and_odd_angle_count(oracle, built_lib):
    # N even (possible with sub-sampling, tv_hpc.F90:555) and T odd (V=1 pairs angles)
    N, T, wpu = 64, 37, 6
    th = syn.angles(T)
    ell = syn.random_ellipses(9, 0.3 * N)
    sino = syn.analytic_sinogram(ell, N, th).numpy().astype(np.float32)
    t = Tomography(N, th, wpu)
    got = t.iradon(torch.from_numpy(sino).cuda())
    assert rel(got, oracle.iradon(sino.astype(np.float64), th, wpu, 64)) < FBP_TOL


def test_empty_batch_and_bad_shapes(case):
    t = Tomography(case["N"], case["th"], case["wpu"])
    out = t.iradon(torch.zeros(0, case["T"], case["N"], device="cuda"))
    assert out.shape == (0, case["N"], case["N"])
    with pytest.raises(ValueError):
        t.iradon(torch.zeros(case["T"] + 1, case["N"], device="cuda"))


def test_projector_variants_agree(case, oracle):
    """The batched single-precision projector variants (pair images; lane
    image + transpose; the same with row-parity loads; the same with reused
    taps) compute the same sums up to summation order, also on random images
    that reach the border."""
    t = Tomography(case["N"], case["th"], case["wpu"])
    t.set_option(8, 0)                     # the reference's single-precision positions
    rng = np.random.default_rng(5)
    for x in (case["img"][:5].astype(np.float32), rng.standard_normal((5, case["N"], case["N"])).astype(np.float32)):
        img = torch.from_numpy(x).cuda()
        outs = []
        for v in range(7):
            t.set_option(7, v)
            outs.append(t.radon(img))
        # reusing the previous sample's taps, skipping steps that cannot meet
        # a valid cell, pairing the FMAs and walking the rays in bands of
        # pixel lines change neither values nor order
        assert all(torch.equal(outs[v], outs[1]) for v in range(3, 7))
        ref = oracle.radon(x, case["th"], 32)
        for o in outs:
            assert rel(o, ref) < 1e-6



def test_exact_positions_backprojection(oracle, built_lib):
    """Option 8 = 1 (the default): backprojection sample positions from the split FP64 angle
    tables, against option 8 = 0.  On a ramp-filtered-like (high-pass) input at a 1025 grid, where
    the reference's single-precision positions are off by ~6e-5 px, the exact
    positions bring the result to single-precision round-off of the FP64
    oracle."""
    N, T, wpu = 1025, 300, 30
    th = syn.angles(T)
    q = np.random.default_rng(11).standard_normal((1, T, N)).astype(np.float32)
    ref64 = oracle.backproject(q.astype(np.float64), th, wpu, 64)
    t = Tomography(N, th, wpu)
    assert t.get_option(8) == 1            # exact positions are the default
    t.set_option(8, 0)
    qc = torch.from_numpy(q).cuda()
    e_ref = rel(t.backproject(qc), ref64)
    t.set_option(8, 1)
    assert t.get_option(8) == 1
    e_exact = rel(t.backproject(qc), ref64)
    assert e_exact < 1e-6 and e_exact < e_ref / 5, (e_exact, e_ref)
    # double precision ignores the option
    assert rel(t.backproject(qc.double()), ref64) < 1e-11


def test_exact_positions_projector_and_adjoint(oracle, built_lib):
    """Option 8 = 1 for the projector variants, the single-slice path and the
    exact adjoint: closer to the FP64 oracle than the reference's
    single-precision positions on a random interior image at a 1025 grid,
    and the adjoint pair still passes the dot-product test."""
    N, T, wpu = 1025, 120, 30
    th = syn.angles(T)
    rng = np.random.default_rng(12)
    x = rng.standard_normal((4, N, N)).astype(np.float32)
    x[:, :3, :] = x[:, -3:, :] = x[:, :, :3] = x[:, :, -3:] = 0
    ref64 = oracle.radon(x.astype(np.float64), th, 64)
    t = Tomography(N, th, wpu)
    t.set_option(8, 0)
    xc = torch.from_numpy(x).cuda()
    e_ref = rel(t.radon(xc), ref64)
    t.set_option(8, 1)
    for proj in (6, 5, 4, 3, 2, 1, 0):
        t.set_option(7, proj)
        e4 = rel(t.radon(xc), ref64)                      # batched, 4 slices per thread
        assert e4 < 3e-6 and e4 < e_ref / 5, (proj, e4, e_ref)
    e1 = rel(t.radon(xc[:1]), ref64[:1])                  # single-slice staggered path
    assert e1 < 3e-6 and e1 < e_ref / 5, e1
    # dot-product test on positive data (no cancellation in either inner product)
    xp = torch.from_numpy(rng.uniform(size=(4, N, N)).astype(np.float32)).cuda()
    y = torch.from_numpy(rng.uniform(size=(4, T, N)).astype(np.float32)).cuda()
    lhs = torch.sum(t.radon(xp).double() * y.double()).item()
    rhs = torch.sum(xp.double() * t.radon_adjoint(y).double()).item()
    assert abs(lhs - rhs) <= 1e-6 * abs(lhs)


@pytest.mark.parametrize("N, T, S, wpu", [(725, 97, 37, 20), (1025, 60, 4, 30), (2049, 24, 33, 100), (64, 37, 9, 6),
                                           (3, 11, 4, 1)])
def test_line_projector_bitwise(N, T, S, wpu):
    """Projector variant 6 (pixel lines of 32 slices, rays walked in bands of
    rows, several bands from N = 725 on) gives bit for bit the sums of
    variant 5, in both position modes, on random images that reach the
    border, with slice counts that leave super-groups partly empty and
    angles on and near the axes."""
    th = np.concatenate([syn.angles(T - 8), [0.0, 45.0, 90.0, 135.0, 180.0, 89.9999, 90.0001, 1e-5]])
    th = th.astype(np.float32)
    t = Tomography(N, th, wpu)
    x = torch.from_numpy(np.random.default_rng(N + S).standard_normal((S, N, N)).astype(np.float32)).cuda()
    for ex in (0, 1):
        t.set_option(8, ex)
        t.set_option(7, 5)
        ref = t.radon(x)
        for v in (6,):
            t.set_option(7, v)
            got = t.radon(x)
            assert torch.equal(got, ref), (ex, v, (got - ref).abs().max().item())


def test_backprojection_groups_per_thread(oracle, built_lib):
    """ACU_OPT_BP_GROUPS: one, two or four 4-slice groups per thread give
    identical images in both position modes (the groups share only the
    angle's table entry and position); the group count need not divide."""
    N, T = 257, 70
    th = syn.angles(T)
    t = Tomography(N, th, 10)
    for S in (16, 20):                 # 4 groups (all counts divide), 5 groups (none does)
        q = torch.randn(S, T, N, device="cuda")
        for ex in (0, 1):
            t.set_option(8, ex)
            outs = []
            for u in (1, 2, 4, 0):
                t.set_option(10, u)
                outs.append(t.backproject(q))
            assert all(torch.equal(outs[0], o) for o in outs[1:])
            assert rel(outs[0], oracle.backproject(q.double().cpu().numpy(), th, 10, 64)) < 1e-5
    with pytest.raises(Exception):
        t.set_option(10, 3)


def test_backprojection_table_in_parameters(built_lib):
    """ACU_OPT_BP_PARAM_TABLE: the backprojection's per-angle table read from
    the launch parameters (T <= 1920) or from device memory gives identical
    images in both position modes; above 1920 angles the device table is
    used."""
    for N, T, S in ((257, 1920, 8), (129, 1921, 8), (257, 90, 4)):
        t = Tomography(N, syn.angles(T), 10)
        q = torch.randn(S, T, N, device="cuda")
        for ex in (1, 0):
            t.set_option(8, ex)
            t.set_option(12, 1)
            a = t.backproject(q)
            t.set_option(12, 0)
            assert torch.equal(a, t.backproject(q))
        t.close()


@pytest.mark.parametrize("N, T, S", [(257, 90, 16), (1025, 300, 8), (64, 37, 4), (3, 7, 4), (129, 1920, 4)])
def test_backprojection_staged_identical(N, T, S):
    """ACU_OPT_BP_STAGED: the sinogram bins each 32x8 tile needs, staged in
    shared memory by bulk copies, give the images of the L1 path bit for bit
    (exact positions), including tiles cut by the grid's edge and angle counts
    that leave the last stage partly filled."""
    t = Tomography(N, syn.angles(T), 10)
    q = torch.randn(S, T, N, device="cuda")
    t.set_option(14, 0)
    ref = t.backproject(q)
    t.set_option(14, 1)
    got = t.backproject(q)
    assert torch.isfinite(got).all()
    assert torch.equal(got, ref), (got - ref).abs().max().item()
    with pytest.raises(Exception):
        t.set_option(14, 2)


@pytest.mark.parametrize("positions", [0, 1])
def test_operators_at_the_2049_grid(oracle, positions):
    """The projector (32 random images) and FBP (32 phantom sinograms) at the
    full 2049 grid (the pixel-line projector, the 4096-point FFT filter and
    the parameter-table backprojection), against the oracle on three of the
    slices: the reference's positions against its single-precision
    restatement, exact positions against FP64.  Seven angles off the grid
    directions keep the oracle's part to seconds."""
    N, T, S, wpu = 2049, 7, 32, 100
    th = (syn.angles(T) + 0.37).astype(np.float32)
    rng = np.random.default_rng(3)
    img = rng.random((S, N, N), dtype=np.float32)
    t = Tomography(N, th, wpu)
    t.set_option(8, positions)
    pick = [0, 13, 31]
    prec = 32 if positions == 0 else 64
    dt = np.float32 if prec == 32 else np.float64
    sino = t.radon(torch.from_numpy(img).cuda()).cpu().numpy()
    ref = oracle.radon(img[pick].astype(dt), th, prec)
    # against FP64 the single-precision sums of ~2000 positive samples per ray
    # carry ~1e-6 of rounding (1.2e-6 measured); against the single-precision
    # restatement the same sums agree far closer
    assert rel(sino[pick], ref) < (1e-6 if prec == 32 else 5e-6)
    # FBP of phantom sinograms (random ellipses), the reconstruction the bar is
    # set for; uniform noise would make the ramp filter's output small against
    # its input and measure single-precision cancellation instead
    phant = np.stack([syn.analytic_sinogram(syn.random_ellipses(100 + k, 0.35 * N), N, th).numpy()
                      for k in range(S)]).astype(np.float32)
    fbp = t.iradon(torch.from_numpy(phant).cuda()).cpu().numpy()
    ref = oracle.iradon(phant[pick].astype(dt), th, wpu, prec)
    assert rel(fbp[pick], ref) < FBP_TOL
    t.close()


@pytest.mark.parametrize("S", [1, 8])
def test_filter_4096_points_against_fp64(oracle, S):
    """The 4096-point filter (grids 1449 to 2049: three radix-16 passes in
    registers) against the oracle's FP64 direct convolution, one slice (two
    columns per transform) and two 4-slice groups (lane layout), with an odd
    angle count leaving the last transform's second column empty."""
    N, T = 2049, 31
    th = syn.angles(T)
    q = np.stack([syn.analytic_sinogram(syn.random_ellipses(40 + k, 0.35 * N), N, th).numpy()
                  for k in range(S)]).astype(np.float32)
    t = Tomography(N, th, 10)
    got = t.filter(torch.from_numpy(q).cuda()).cpu().numpy()
    ref = oracle.filter_rows(q.astype(np.float64), 64)
    assert rel(got, ref) < 3e-5
    t.close()
