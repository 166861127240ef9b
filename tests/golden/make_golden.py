"""Writes the golden fixture of the single-slice split-Bregman TV
configuration: a 1449^2 grid (1448 detector bins made odd), 900 angles over
[0, 180), Poisson counts at I0 = 5e3 of a seeded 10-ellipse phantom whose
support is the 1024-pixel disc, lambda = 0.05, mu = 1.0, wpu = 100,
50 Bregman outer x 10 CG iterations (tomography/tv_hpc.F90:162-363).

The fixture holds the counts (uint16) and the CPU oracle's TV results in the
reference's single precision (source operation order, single-precision
reductions: the reference's own CPU arithmetic) and in double precision
(stored rounded to float32).  The normalised sinogram the solvers see is
p = -log(counts / I0), evaluated in double and rounded to float32, so that it
is the same on every machine.

Run once on a CPU (about 2 hours on 8 cores; the oracle parallelises over
rows with OpenMP, which does not change its results):
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

N, T, I0, SEED = 1449, 900, 5e3, 2
LAM, MU, WPU, NINNER, NOUTER, NCG = 0.05, 1.0, 100, 1, 50, 10
OUT = os.path.join(HERE, "tv_1449sq_900ang.npz")


def angles():
    return (np.arange(T, dtype=np.float64) * (180.0 / T)).astype(np.float32)


def counts():
    """Poisson counts I0 exp(-p) of the analytic projections p of the phantom."""
    from acumen_gb300 import synthetic as syn
    ell = syn.random_ellipses(SEED, 512.0)
    p = syn.analytic_sinogram(ell, N, angles()).numpy()
    rng = np.random.default_rng(SEED)
    c = rng.poisson(I0 * np.exp(-p))
    return np.clip(c, 1, 65535).astype(np.uint16)


def normalised(c):
    """The reference's log-normalisation with a noise-free flat field
    (tomography/fits_to_hpc.F90:243), in double, rounded to float32."""
    return (-np.log(c.astype(np.float64) / max(I0, 1.0))).astype(np.float32)


def main():
    from oracle import oracle as O
    c = counts()
    f = normalised(c)
    th = angles()
    res = {}
    for prec, red in ((64, 1), (32, 0)):
        t0 = time.time()
        tv, _ = O.tvopt(f.astype(np.float64 if prec == 64 else np.float32), th, WPU, NINNER, NOUTER, NCG,
                        LAM, MU, prec=prec, red_mode=red)
        res[prec] = tv.astype(np.float32)
        print(f"oracle FP{prec}: {time.time() - t0:.0f} s", flush=True)
    np.savez_compressed(OUT, counts=c, theta=th, tv_f32=res[32], tv_f64=res[64],
                        params=np.array([N, T, I0, LAM, MU, WPU, NINNER, NOUTER, NCG], np.float64))
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
