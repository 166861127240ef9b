"""Ragged batches (64-problem shape scaled down): problems of different grid
side and angle count in one batch, each checked against the oracle.

Tolerances as the uniform path: radon 1e-6, iradon 1e-5 (relative L2, FP64
oracle), TV 1e-4 inside the reconstruction disc against the FP64 oracle.
"""
import numpy as np
import pytest

from acumen_gb300 import synthetic as syn
from acumen_gb300.batch import RaggedBatch

pytestmark = pytest.mark.gpu


def rel(a, b, m=None):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    if m is not None:
        a, b = a[m], b[m]
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def probs(built_lib):
    rng = np.random.default_rng(4)
    sides = [33, 97, 49, 65, 129, 41]
    Ts = [int(rng.integers(20, 90)) for _ in sides]
    thetas = [syn.angles(T) for T in Ts]
    imgs = [syn.rasterize(syn.random_ellipses(40 + i, 0.3 * N), N).numpy() for i, N in enumerate(sides)]
    sinos = [syn.analytic_sinogram(syn.random_ellipses(40 + i, 0.3 * N), N, th).numpy()
             for i, (N, th) in enumerate(zip(sides, thetas))]
    return dict(N=sides, T=Ts, th=thetas, imgs=imgs, sinos=sinos, wpu=4)


def test_batch_operators_match_oracle(probs, oracle):
    b = RaggedBatch(probs["N"], probs["th"], probs["wpu"])
    r = b.radon(probs["imgs"])
    for i, (img, th) in enumerate(zip(probs["imgs"], probs["th"])):
        assert rel(r[i], oracle.radon(img, th, 64)) < 1e-6, i
    ir = b.iradon(probs["sinos"])
    for i, (s, th) in enumerate(zip(probs["sinos"], probs["th"])):
        assert rel(ir[i], oracle.iradon(s, th, probs["wpu"], 64)) < 1e-5, i
    w, rows = b.tuning()
    assert w in (2, 4, 8, 16) and rows in (4, 8, 16)


def test_batch_tv_matches_oracle(probs, oracle):
    b = RaggedBatch(probs["N"], probs["th"], probs["wpu"])
    tv, fbp = b.tvopt(probs["sinos"], 1, 4, 4, 0.05, 1.0)
    for i, (s, th, N) in enumerate(zip(probs["sinos"], probs["th"], probs["N"])):
        ref_tv, ref_fbp = oracle.tvopt(s, th, probs["wpu"], 1, 4, 4, 0.05, 1.0, prec=64)
        mask = oracle.cmask(N, len(th), probs["wpu"], 64) > 0
        assert rel(fbp[i], ref_fbp) < 1e-5, i
        assert rel(tv[i], ref_tv, mask) < 1e-4, i
    # a second solve reuses the captured graph and gives the same result
    tv2, _ = b.tvopt(probs["sinos"], 1, 4, 4, 0.05, 1.0)
    for a, c in zip(tv, tv2):
        np.testing.assert_array_equal(a, c)


def test_batch_exact_positions(probs, oracle):
    """ACU_OPT_POSITIONS on a ragged batch: the projector gives exactly what
    the uniform single-slice path gives with the same option, both operators
    stay within their bars of the FP64 oracle, and TV within 1e-4."""
    from acumen_gb300.tomography import Tomography
    b = RaggedBatch(probs["N"], probs["th"], probs["wpu"])
    b.set_option(8, 1)
    with pytest.raises(Exception):
        b.set_option(1, 0)
    r = b.radon(probs["imgs"])
    ir = b.iradon(probs["sinos"])
    for i, (img, s, th, N) in enumerate(zip(probs["imgs"], probs["sinos"], probs["th"], probs["N"])):
        t = Tomography(N, th, probs["wpu"])
        t.set_option(8, 1)
        np.testing.assert_array_equal(r[i], t.radon(img.astype(np.float32)))
        assert rel(r[i], oracle.radon(img, th, 64)) < 1e-6, i
        assert rel(ir[i], t.iradon(s.astype(np.float32))) < 1e-6, i
        assert rel(ir[i], oracle.iradon(s, th, probs["wpu"], 64)) < 1e-5, i
        t.close()
    tv, _ = b.tvopt(probs["sinos"], 1, 4, 4, 0.05, 1.0)
    for i, (s, th, N) in enumerate(zip(probs["sinos"], probs["th"], probs["N"])):
        ref_tv, _ = oracle.tvopt(s, th, probs["wpu"], 1, 4, 4, 0.05, 1.0, prec=64)
        mask = oracle.cmask(N, len(th), probs["wpu"], 64) > 0
        assert rel(tv[i], ref_tv, mask) < 1e-4, i


def test_batch_radon_refresh(probs, oracle):
    """ACU_OPT_RADON_REFRESH on a ragged batch: radon(uk) carried through the
    CG updates (default, recomputed every fifth outer iteration) against the
    reference's recomputation every outer iteration."""
    args = (probs["sinos"], 1, 6, 4, 0.05, 1.0)
    b = RaggedBatch(probs["N"], probs["th"], probs["wpu"])
    tv5, _ = b.tvopt(*args)
    b.set_option(11, 1)
    tv1, _ = b.tvopt(*args)
    b.set_option(11, 0)
    tv0, _ = b.tvopt(*args)
    for i, (s, th, N) in enumerate(zip(probs["sinos"], probs["th"], probs["N"])):
        mask = oracle.cmask(N, len(th), probs["wpu"], 64) > 0
        ref_tv, _ = oracle.tvopt(s, th, probs["wpu"], 1, 6, 4, 0.05, 1.0, prec=64)
        for tv in (tv5, tv1, tv0):
            assert rel(tv[i], ref_tv, mask) < 1e-4, i
        assert rel(tv5[i], tv1[i], mask) < 2e-5, i
    with pytest.raises(Exception):
        b.set_option(11, -1)


def test_batch_at_uneven_batch_sizes_vs_fp64_oracle(oracle, built_lib):
    """Problems of the 64-problem configuration's sizes (sides 256 and 512:
    grids 363 and 725, the 180-1500 angle range) in one ragged batch, one
    outer iteration of 10 CG steps, against the FP64 oracle inside the disc."""
    rng = np.random.default_rng(64)
    spec = [(363, 1500), (725, 240), (363, 180)]
    ths = [syn.angles(T) for _, T in spec]
    sinos = [syn.analytic_sinogram(syn.random_ellipses(80 + i, 0.35 * N), N, th).numpy()
             + 1e-3 * rng.standard_normal((len(th), N)) for i, ((N, _), th) in enumerate(zip(spec, ths))]
    b = RaggedBatch([N for N, _ in spec], ths, 100)
    tv, fbp = b.tvopt(sinos, 1, 1, 10, 0.05, 1.0)
    for i, ((N, T), th, f) in enumerate(zip(spec, ths, sinos)):
        ref_tv, ref_fbp = oracle.tvopt(f, th, 100, 1, 1, 10, 0.05, 1.0, prec=64)
        mask = oracle.cmask(N, T, 100, 64) > 0
        assert rel(fbp[i], ref_fbp) < 1e-5, i
        assert rel(tv[i], ref_tv, mask) < 1e-4, i
