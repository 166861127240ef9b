"""The algebra behind ACU_OPT_RESIDUAL = 2 on the CPU, with the oracle's FP64
operators (tomography/tv_hpc.F90:84-159): the initial CG residual's
backprojection iradon(fk - radon(uk)) equals bd + dacc, where
bd = iradon(f - radon(uk)) follows every uk += alpha p as bd -= alpha
iradon(radon(p)) and dacc = iradon(fk - f) gains bd at every Bregman update
fk += f - radon(uk).  Replayed over a few outer iterations of random CG-like
updates, the carried pair stays within FP64 round-off of the direct form."""
import numpy as np

from acumen_gb300 import synthetic as syn


def test_carried_backprojection_identity(oracle):
    N, T, wpu = 33, 24, 4
    th = syn.angles(T)
    rng = np.random.default_rng(7)
    f = rng.random((T, N))
    uk = oracle.iradon(f, th, wpu, 64)
    fk = f.copy()
    ruk = oracle.radon(uk, th, 64)
    bd = oracle.iradon(f - ruk, th, wpu, 64)
    dacc = np.zeros((N, N))
    for outer in range(4):
        for cg in range(5):
            p = rng.standard_normal((N, N))
            alpha = rng.uniform(0.01, 0.2)
            rp = oracle.radon(p, th, 64)
            irpt = oracle.iradon(rp, th, wpu, 64)
            uk = uk + alpha * p
            ruk = ruk + alpha * rp               # radon(uk) carried
            bd = bd - alpha * irpt               # iradon(f - radon(uk)) carried
            direct = oracle.iradon(fk - ruk, th, wpu, 64)
            np.testing.assert_allclose(bd + dacc, direct, rtol=0, atol=1e-10 * np.abs(direct).max())
        fk = fk + f - ruk                        # Bregman update
        dacc = dacc + bd                         # iradon(fk - f) gains iradon(f - radon(uk))
        direct = oracle.iradon(fk - ruk, th, wpu, 64)
        np.testing.assert_allclose(bd + dacc, direct, rtol=0, atol=1e-10 * np.abs(direct).max())
