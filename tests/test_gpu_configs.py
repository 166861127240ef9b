"""Parity at the benchmark configurations' full sizes, through the C ABI.

FBP (tomography/tv_hpc.F90:84-126), one 725^2 slice (724 bins made odd) at
720 angles over [0, 180), from Poisson counts at I0 = flat = 1e4 with
dark = 100, normalised in both of the reference's modes
(tomography/fits_to_hpc.F90:243 and :244).  Bars (relative L2, full grid and
the centred 512^2 crop):
  - exact positions (the default) against the FP64 oracle: <= 1e-5;
  - the reference's single-precision positions against the oracle's
    single-precision restatement (the reference's own CPU arithmetic): <= 1e-5.

Split-Bregman TV (tomography/tv_hpc.F90:162-363), one 1449^2 slice at 900
angles, lambda = 0.05, mu = 1, 50 outer x 10 CG iterations, against the
committed golden fixture of the CPU oracle in FP64 and in the reference's
single precision (tests/golden/make_golden.py).  Bars inside the
reconstruction disc (mask > 0; outside it the reference's normal operator
reduces to lambda times the periodic Laplacian, nearly singular, where the
oracle's own single-precision run departs from its FP64 run):
  - exact positions against the FP64 oracle: <= 1e-4 (full image < 2e-3);
  - the reference's positions against the oracle's single precision: <= 1e-4.
"""
import os
import sys

import numpy as np
import pytest
import torch

from acumen_gb300 import synthetic as syn
from acumen_gb300.tomography import Tomography

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = {k: os.path.join(HERE, "golden", f"tv_1449sq_900ang_{k}.npz") for k in ("input", "fp64", "fp32")}


def rel(a, b, m=None):
    a = np.asarray(a.cpu() if isinstance(a, torch.Tensor) else a, np.float64)
    b = np.asarray(b.cpu() if isinstance(b, torch.Tensor) else b, np.float64)
    if m is not None:
        a, b = a[..., m], b[..., m]
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def crop512(a, N=725):
    o = (N - 512) // 2
    return np.asarray(a)[..., o:o + 512, o:o + 512]


@pytest.fixture(scope="module")
def fbp_case(built_lib, oracle):
    th, ell, counts, flat, dark = syn.counts_sinogram_725(seed=1)
    c = counts.numpy().astype(np.float32)
    ob = np.full(c.shape, flat, np.float32)      # the flat and dark level of every detector reading
    df = np.full(c.shape, dark, np.float32)
    return dict(th=th, p={m: oracle.normalize(c, ob, df, m) for m in (0, 1)})


@pytest.mark.parametrize("norm_mode", [0, 1])
def test_fbp_725sq_720ang(fbp_case, oracle, norm_mode):
    N, wpu = 725, 100
    th, p = fbp_case["th"], fbp_case["p"][norm_mode]
    ref64 = oracle.iradon(p.astype(np.float64), th, wpu, 64)
    ref32 = oracle.iradon(p, th, wpu, 32)
    t = Tomography(N, th, wpu)
    assert t.get_option(8) == 1
    ex = t.iradon(torch.from_numpy(p[None]).cuda()).cpu().numpy()[0]
    assert rel(ex, ref64) <= 1e-5 and rel(crop512(ex), crop512(ref64)) <= 1e-5
    t.set_option(8, 0)
    rp = t.iradon(torch.from_numpy(p[None]).cuda()).cpu().numpy()[0]
    assert rel(rp, ref32) <= 1e-5 and rel(crop512(rp), crop512(ref32)) <= 1e-5
    # host-buffer entry point (get_slice's form) gives the same image
    np.testing.assert_array_equal(t.iradon(p[None])[0], rp)
    t.close()


@pytest.fixture(scope="module")
def tv_case(built_lib):
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_golden as mg
    z = np.load(GOLDEN["input"])
    assert int(z["params"][0]) == mg.N and int(z["params"][1]) == mg.T
    f = mg.normalised(z["counts"])
    ref = {k: np.load(GOLDEN[k])["tv"] if os.path.exists(GOLDEN[k]) else None for k in ("fp64", "fp32")}
    return dict(mg=mg, f=f, th=z["theta"], tv32=ref["fp32"], tv64=ref["fp64"])


def _solve(case, positions, plain=False):
    mg = case["mg"]
    t = Tomography(mg.N, case["th"], mg.WPU)
    t.set_option(8, positions)
    tv, fbp = t.tvopt(torch.from_numpy(case["f"][None]).cuda(), mg.NINNER, mg.NOUTER, mg.NCG, mg.LAM, mg.MU,
                      plain=plain)
    t.close()
    return tv.cpu().numpy()[0]


def test_tv_1449sq_900ang_exact_positions_vs_fp64_golden(tv_case, oracle):
    if tv_case["tv64"] is None:
        pytest.skip("golden FP64 result not generated")
    mg = tv_case["mg"]
    mask = oracle.cmask(mg.N, mg.T, mg.WPU, 64) > 0
    tv = _solve(tv_case, 1)
    assert rel(tv, tv_case["tv64"], mask) <= 1e-4
    assert rel(tv, tv_case["tv64"]) < 2e-3


def test_tv_1449sq_900ang_reference_positions_vs_fp32_golden(tv_case, oracle):
    if tv_case["tv32"] is None:
        pytest.skip("golden FP32 result not generated")
    mg = tv_case["mg"]
    mask = oracle.cmask(mg.N, mg.T, mg.WPU, 64) > 0
    for plain in (False, True):
        tv = _solve(tv_case, 0, plain)
        assert rel(tv, tv_case["tv32"], mask) <= 1e-4, plain
