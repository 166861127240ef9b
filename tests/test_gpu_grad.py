"""Gradient of the registration-aware TV objective (the differentiable path): the hand-written adjoint kernels against central finite differences
(h = 1e-3) and against the FP64 oracle gradient (oracle/acumen_oracle.c
orc_tv_loss_grad_f64).

Tolerances: FP64 kernels vs FP64 oracle 1e-10 (relative L2, gradient and
loss); FP32 kernels vs FP64 oracle 1e-5; finite differences of the FP64
loss vs its analytic gradient: 1e-4 per image coordinate (the objective is
smooth in u), 1% of the gradient's RMS per angle offset (piecewise smooth in
the offsets, see the test).
"""
import numpy as np
import pytest
import torch

from acumen_gb300 import synthetic as syn
from acumen_gb300.autograd import tv_objective
from acumen_gb300.tomography import Tomography

pytestmark = pytest.mark.gpu

LAM, EPS = 0.05, 0.05


def rel(a, b):
    a = np.asarray(a.cpu() if isinstance(a, torch.Tensor) else a, np.float64)
    b = np.asarray(b.cpu() if isinstance(b, torch.Tensor) else b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def prob(built_lib, oracle):
    N, T = 49, 36
    th = syn.angles(T)
    S = 2
    rng = np.random.default_rng(0)
    u = np.stack([syn.rasterize(syn.random_ellipses(20 + s, 0.3 * N), N).numpy() for s in range(S)])
    u += 0.01 * rng.standard_normal(u.shape)
    off = rng.normal(0, 2.0, (S, T))
    y = np.stack([syn.analytic_sinogram(syn.random_ellipses(30 + s, 0.3 * N), N, th).numpy() for s in range(S)])
    ref = [oracle.tv_loss_grad(u[s], off[s], y[s], th, LAM, EPS) for s in range(S)]
    return dict(N=N, T=T, th=th, u=u, off=off, y=y, S=S,
                loss=np.array([r[0] for r in ref]), gu=np.stack([r[1] for r in ref]),
                go=np.stack([r[2] for r in ref]))


def test_f64_gradient_matches_fp64_oracle(prob):
    t = Tomography(prob["N"], prob["th"], 4)
    loss, gu, go = t.tv_loss_grad(torch.from_numpy(prob["u"]).cuda(), torch.from_numpy(prob["off"]).cuda(),
                                  torch.from_numpy(prob["y"]).cuda(), LAM, EPS)
    np.testing.assert_allclose(loss, prob["loss"], rtol=1e-11)
    assert rel(gu, prob["gu"]) < 1e-10
    assert rel(go, prob["go"]) < 1e-10


def test_f32_gradient_matches_fp64_oracle(prob):
    t = Tomography(prob["N"], prob["th"], 4)
    cu = lambda a: torch.from_numpy(a.astype(np.float32)).cuda()
    loss, gu, go = t.tv_loss_grad(cu(prob["u"]), cu(prob["off"]), cu(prob["y"]), LAM, EPS)
    np.testing.assert_allclose(loss, prob["loss"], rtol=1e-5)
    assert rel(gu, prob["gu"]) < 1e-5
    assert rel(go, prob["go"]) < 1e-4


def test_zero_offsets_equal_plain_projector(prob):
    t = Tomography(prob["N"], prob["th"], 4)
    u = torch.from_numpy(prob["u"]).cuda()
    y = torch.zeros(prob["S"], prob["T"], prob["N"], dtype=torch.float64, device="cuda")
    loss, _, _ = t.tv_loss_grad(u, torch.zeros(prob["S"], prob["T"], dtype=torch.float64, device="cuda"), y, 0.0, EPS)
    ru = t.radon(u)
    np.testing.assert_allclose(loss, 0.5 * (ru ** 2).sum(dim=(1, 2)).cpu().numpy(), rtol=1e-12)


def test_autograd_wrapper_finite_differences(prob):
    t = Tomography(prob["N"], prob["th"], 4)
    u = torch.from_numpy(prob["u"]).cuda().requires_grad_(True)
    off = torch.from_numpy(prob["off"]).cuda().requires_grad_(True)
    y = torch.from_numpy(prob["y"]).cuda()
    L = tv_objective(t, u, off, y, LAM, EPS)
    L.backward()
    h = 1e-3
    rng = np.random.default_rng(1)

    def f(uu, oo):
        with torch.no_grad():
            return float(tv_objective(t, uu, oo, y, LAM, EPS))

    checked = 0
    # image coordinates inside the support
    for _ in range(12):
        s, i, j = rng.integers(0, prob["S"]), rng.integers(12, prob["N"] - 12), rng.integers(12, prob["N"] - 12)
        up, um = u.detach().clone(), u.detach().clone()
        up[s, i, j] += h
        um[s, i, j] -= h
        fd = (f(up, off.detach()) - f(um, off.detach())) / (2 * h)
        g = float(u.grad[s, i, j])
        assert abs(fd - g) <= 1e-4 * max(1.0, abs(g)), (s, i, j, fd, g)
        checked += 1
    assert checked == 12


def test_offset_gradient_finite_differences(prob):
    """The projector is bilinear, so the objective is only piecewise smooth in
    the offsets: each sample whose +-h move crosses a cell edge adds a small
    derivative jump.  On a smooth image these stay below 1% of the gradient's
    RMS, which is the bound here; the exact check of the same gradient is the
    1e-10 agreement with the FP64 oracle above."""
    N, T, S = prob["N"], prob["T"], 1
    t = Tomography(N, prob["th"], 4)
    j = np.arange(1, N + 1) - (N + 1) // 2
    Y, X = np.meshgrid(j, j, indexing="ij")
    u = np.exp(-((X - 3.0) ** 2 + (Y + 2.0) ** 2) / (2 * 6.0 ** 2))[None] + \
        0.5 * np.exp(-((X + 7.0) ** 2 + (Y - 5.0) ** 2) / (2 * 4.0 ** 2))[None]
    rng = np.random.default_rng(3)
    off = torch.from_numpy(rng.normal(0, 2.0, (S, T))).cuda().requires_grad_(True)
    ut = torch.from_numpy(u).cuda().requires_grad_(True)
    y = torch.from_numpy(prob["y"][:1]).cuda()
    L = tv_objective(t, ut, off, y, LAM, EPS)
    L.backward()
    g = off.grad.cpu().numpy()[0]
    scale = float(np.sqrt(np.mean(g ** 2)))
    h = 1e-3
    for k in rng.choice(T, 12, replace=False):
        op, om = off.detach().clone(), off.detach().clone()
        op[0, k] += h
        om[0, k] -= h
        with torch.no_grad():
            fd = (float(tv_objective(t, ut.detach(), op, y, LAM, EPS)) -
                  float(tv_objective(t, ut.detach(), om, y, LAM, EPS))) / (2 * h)
        assert abs(fd - g[k]) <= 1e-2 * scale, (k, fd, g[k], scale)
