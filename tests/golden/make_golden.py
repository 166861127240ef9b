"""Writes the golden fixture of the single-slice split-Bregman TV
configuration: a 1449^2 grid (1448 detector bins made odd), 900 angles over
[0, 180), Poisson counts at I0 = 5e3 of a seeded 10-ellipse phantom whose
support is the 1024-pixel disc, lambda = 0.05, mu = 1.0, wpu = 100,
50 Bregman outer x 10 CG iterations (tomography/tv_hpc.F90:162-363).

The fixture is three files: the counts (uint16) with the angles and
parameters, and the CPU oracle's TV result in double precision (stored
rounded to float32) and in the reference's single precision (source operation
order, single-precision reductions: the reference's own CPU arithmetic).  The normalised sinogram the solvers see is
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
INPUT = os.path.join(HERE, "tv_1449sq_900ang_input.npz")
RESULT = {64: os.path.join(HERE, "tv_1449sq_900ang_fp64.npz"), 32: os.path.join(HERE, "tv_1449sq_900ang_fp32.npz")}


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


def main(precisions=(64, 32)):
    """Writes the input file, then one result file per precision as each
    solve finishes (FP64 first)."""
    from oracle import oracle as O
    c = counts()
    f = normalised(c)
    th = angles()
    np.savez_compressed(INPUT, counts=c, theta=th,
                        params=np.array([N, T, I0, LAM, MU, WPU, NINNER, NOUTER, NCG], np.float64))
    for prec in precisions:
        red = 1 if prec == 64 else 0
        t0 = time.time()
        tv, _ = O.tvopt(f.astype(np.float64 if prec == 64 else np.float32), th, WPU, NINNER, NOUTER, NCG,
                        LAM, MU, prec=prec, red_mode=red)
        np.savez_compressed(RESULT[prec], tv=tv.astype(np.float32))
        print(f"oracle FP{prec}: {time.time() - t0:.0f} s, wrote {RESULT[prec]}", flush=True)


if __name__ == "__main__":
    main()
