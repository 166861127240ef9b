"""Seeded synthetic inputs in the reference's geometry.

The reference's neutron-CT datasets are not available; these generators stand
in for them with the shapes and value ranges of the benchmark configurations:
random-ellipse phantoms, their analytic parallel-beam projections in the
projector's own convention (tomography/tv_hpc.F90:137-156), Poisson counts
with flat/dark frames, and raw uint16 projection stacks with a rotation-axis
offset.  Everything is computed with torch so that large stacks can be made
directly on the GPU; small cases run on the CPU.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import torch


@dataclass
class Ellipse:
    cx: float   # centre relative to the grid midpoint, pixels
    cy: float
    a: float    # semi-axes, pixels
    b: float
    phi: float  # rotation, radians
    v: float    # attenuation


def random_ellipses(seed: int, radius: float, n: int = 10):
    """Ten (by default) ellipses: centres uniform in the disc of `radius`,
    semi-axes 0.05-0.4 of the radius, attenuation 0.1-1.0."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        while True:
            cx, cy = rng.uniform(-radius, radius, 2)
            if cx * cx + cy * cy < radius * radius:
                break
        a, b = rng.uniform(0.05, 0.4, 2) * radius
        out.append(Ellipse(float(cx), float(cy), float(a), float(b),
                           float(rng.uniform(0, math.pi)), float(rng.uniform(0.1, 1.0))))
    return out


def midpoint(N: int) -> int:
    return (N + 1) // 2


def rasterize(ellipses, N: int, device="cpu", dtype=torch.float64):
    """Phantom image img[jy-1, jx-1] sampled at pixel centres."""
    m = midpoint(N)
    j = torch.arange(1, N + 1, device=device, dtype=dtype) - m
    Y, X = torch.meshgrid(j, j, indexing="ij")
    img = torch.zeros(N, N, device=device, dtype=dtype)
    for e in ellipses:
        c, s = math.cos(e.phi), math.sin(e.phi)
        dx, dy = X - e.cx, Y - e.cy
        u = (c * dx + s * dy) / e.a
        v = (-s * dx + c * dy) / e.b
        img += torch.where(u * u + v * v <= 1.0, e.v, 0.0)
    return img


def analytic_sinogram(ellipses, N: int, theta_deg, det_offset=0.0, device="cpu",
                      dtype=torch.float64, nbins=None):
    """sino[t, jbin-1] = (1/N) * line integral of the phantom along the ray the
    projector samples for bin jbin at angle theta: direction (cos c, sin c)
    through midpoint + (jbin - m + det_offset) * (-sin c, cos c), with
    c = pi*(theta-90)/180.  det_offset (pixels) moves the rotation axis."""
    nb = N if nbins is None else nbins
    m = midpoint(N)
    th = torch.as_tensor(np.asarray(theta_deg, dtype=np.float64), device=device, dtype=dtype)
    ct = math.pi * (th - 90.0) / 180.0
    c, s = torch.cos(ct)[:, None], torch.sin(ct)[:, None]
    jb = torch.arange(1, nb + 1, device=device, dtype=dtype)[None, :]
    off = jb - m - det_offset
    px, py = -s * off, c * off          # ray point relative to the midpoint
    dx, dy = c.expand_as(px), s.expand_as(py)
    out = torch.zeros(len(th), nb, device=device, dtype=dtype)
    for e in ellipses:
        cp, sp = math.cos(e.phi), math.sin(e.phi)
        qx = cp * (px - e.cx) + sp * (py - e.cy)
        qy = -sp * (px - e.cx) + cp * (py - e.cy)
        ex = cp * dx + sp * dy
        ey = -sp * dx + cp * dy
        A = ex * ex / e.a ** 2 + ey * ey / e.b ** 2
        B = 2.0 * (qx * ex / e.a ** 2 + qy * ey / e.b ** 2)
        C = qx * qx / e.a ** 2 + qy * qy / e.b ** 2 - 1.0
        disc = B * B - 4.0 * A * C
        out += e.v * torch.where(disc > 0, torch.sqrt(disc.clamp_min(0)) / A, 0.0)
    return out / N


def angles(T: int, closed: bool = False):
    """T angles evenly over [0,180) (closed=False) or [0,180] (closed=True),
    as the single-precision values theta.dat would hold."""
    if closed:
        return (np.arange(T, dtype=np.float64) * (180.0 / (T - 1))).astype(np.float32)
    return (np.arange(T, dtype=np.float64) * (180.0 / T)).astype(np.float32)


def noisy_counts(sino, I0: float, flat: float, dark: float, seed: int):
    """Poisson(I0 * exp(-p * N_scale)) + dark detector counts for a sinogram
    p (torch).  Returns float32 counts and the (noise-free) flat/dark levels."""
    g = torch.Generator(device=sino.device)
    g.manual_seed(seed)
    lam = (I0 * torch.exp(-sino.double())).float()
    counts = torch.poisson(lam, generator=g) + dark
    return counts, flat + dark, dark


def normalised_sinogram(ellipses, N, theta, I0, seed, flat=None, dark=0.0, mode=0,
                        device="cpu"):
    """Analytic projections -> Poisson counts -> the reference's
    log-normalisation (mode 0: -log(I/max(OB,1)); mode 1: flat/dark form)."""
    p = analytic_sinogram(ellipses, N, theta, device=device)
    counts, ob, df = noisy_counts(p, I0, I0 if flat is None else flat, dark, seed)
    if mode == 0:
        return (-torch.log(counts / max(ob, 1.0))).float()
    return (-torch.log(torch.clamp(counts - df, min=1e-16) / max(ob - df, 1.0))).float()


def counts_sinogram_725(seed=1, device="cpu"):
    """Plain FBP: 10 ellipses in the 512-pixel disc on the 725 grid, 720 angles
    over [0,180), Poisson counts at I0 = flat = 1e4 with dark = 100."""
    N, T = 725, 720
    th = angles(T)
    ell = random_ellipses(seed, 256.0)
    p = analytic_sinogram(ell, N, th, device=device)
    g = torch.Generator(device=p.device)
    g.manual_seed(seed)
    counts = torch.poisson((1e4 * torch.exp(-p)).float(), generator=g) + 100.0
    flat, dark = 1e4 + 100.0, 100.0
    return th, ell, counts, flat, dark


def projection_stack(nproj, ndet, nrows, axis_offset, seed, I0=1e4, dark=100.0,
                     nflat=10, ndark=10, device="cpu"):
    """Raw uint16 projections [nproj][nrows][ndet] of a random-ellipsoid
    volume over angles [0,180] inclusive, with the rotation axis displaced by
    `axis_offset` detector pixels, plus flat and dark stacks.  Row r of every
    projection is the parallel-beam projection of slice r."""
    rng = np.random.default_rng(seed)
    th = angles(nproj, closed=True)
    R = 0.35 * ndet
    ells = []
    for _ in range(10):
        while True:
            cx, cy = rng.uniform(-R, R, 2)
            if cx * cx + cy * cy < R * R:
                break
        a, b = rng.uniform(0.05, 0.4, 2) * R
        cz, hz = rng.uniform(0.2, 0.8) * nrows, rng.uniform(0.2, 0.6) * nrows
        ells.append((cx, cy, a, b, rng.uniform(0, math.pi), rng.uniform(0.1, 1.0), cz, hz))
    Ng = ndet + (1 if ndet % 2 == 0 else 0)
    proj = torch.zeros(nproj, nrows, ndet, device=device, dtype=torch.float32)
    for r in range(nrows):
        el = []
        for (cx, cy, a, b, phi, v, cz, hz) in ells:
            z = (r - cz) / hz
            if abs(z) < 1.0:
                f = math.sqrt(1.0 - z * z)
                el.append(Ellipse(cx, cy, a * f, b * f, phi, v))
        if el:
            p = analytic_sinogram(el, Ng, th, det_offset=axis_offset, device=device, nbins=ndet)
            proj[:, r, :] = (p * Ng / ndet * 4.0).float()
    g = torch.Generator(device=proj.device)
    g.manual_seed(seed)
    raw = torch.poisson((I0 * torch.exp(-proj.double())).float(), generator=g) + dark
    flats = torch.poisson(torch.full((nflat, nrows, ndet), I0, device=device), generator=g) + dark
    darks = torch.poisson(torch.full((ndark, nrows, ndet), dark, device=device), generator=g)
    clamp = lambda x: torch.clamp(x, 0, 65535).to(torch.int32).to(torch.uint16) \
        if hasattr(torch, "uint16") else torch.clamp(x, 0, 65535).to(torch.int32)
    return th, clamp(raw), clamp(flats), clamp(darks)
