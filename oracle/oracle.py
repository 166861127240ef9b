"""ctypes front end of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline / reference legs of bench.py, as the checker or the timed CPU
baseline.  The product package never imports this module.

Array conventions: numpy C-order arrays whose last axis is the reference's
first (fastest) Fortran index, i.e. ``img[..., jy-1, jx-1]`` and
``sino[..., jtheta-1, jbin-1]``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None

_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_c_int, _c_long, _c_float, _c_double = ctypes.c_int, ctypes.c_long, ctypes.c_float, ctypes.c_double


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile (gcc, no GPU)."""
    if force or not os.path.exists(_LIB_PATH) or (
        os.path.getmtime(_LIB_PATH) < max(os.path.getmtime(os.path.join(_HERE, f))
                                          for f in ("acumen_oracle.c", "oracle_impl.h", "Makefile"))):
        subprocess.run(["make", "-B", "-s", "-C", _HERE, "liboracle.so"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        for sfx, p, real in (("f32", _f32p, _c_float), ("f64", _f64p, _c_double)):
            getattr(L, f"orc_filter_taps_{sfx}").argtypes = [_c_int, p]
            getattr(L, f"orc_cmask_{sfx}").argtypes = [_c_int, _c_int, _c_int, p]
            getattr(L, f"orc_filter_{sfx}").argtypes = [_c_int, _c_int, _c_int, p, p]
            getattr(L, f"orc_backproject_{sfx}").argtypes = [_c_int, _c_int, _f32p, _c_int, _c_int, p, p]
            getattr(L, f"orc_iradon_{sfx}").argtypes = [_c_int, _c_int, _f32p, _c_int, _c_int, p, p]
            getattr(L, f"orc_radon_{sfx}").argtypes = [_c_int, _c_int, _f32p, _c_int, p, p]
            getattr(L, f"orc_radon_adjoint_{sfx}").argtypes = [_c_int, _c_int, _f32p, _c_int, p, p]
            getattr(L, f"orc_tvopt_{sfx}").argtypes = [_c_int, _c_int, _f32p, _c_int, _c_int, p,
                                                       _c_int, _c_int, _c_int, real, real, _c_int, p,
                                                       ctypes.c_void_p]
            getattr(L, f"orc_cg_step_{sfx}").argtypes = [_c_int, _c_int, _f32p, _c_int, real, real, _c_int,
                                                         p, p, p, p, p, p, _c_double]
            getattr(L, f"orc_cg_step_{sfx}").restype = _c_double
        L.orc_frame_average.argtypes = [_c_int, _c_long, _f32p, _f32p]
        L.orc_normalize.argtypes = [_c_int, _c_long, _f32p, _f32p, _f32p, _f32p]
        L.orc_minloc_abs.argtypes = [_c_int, _f32p, _c_float]
        L.orc_minloc_abs.restype = _c_int
        L.orc_pick_angle.argtypes = [_c_int, _f32p, _c_long, _f32p, _c_float, _f32p]
        L.orc_resample.argtypes = [_c_int, _c_int, _f32p, _c_float, _c_float, _f32p]
        L.orc_register.argtypes = [_c_int, _c_int, _f32p, _f32p, _c_int,
                                   ctypes.POINTER(_c_float), ctypes.POINTER(_c_float),
                                   ctypes.POINTER(_c_int)]
        L.orc_median27.argtypes = [_c_int, _c_int, _f32p, _f32p, _f32p, _f32p]
        L.orc_proj_to_sino.argtypes = [_c_int, _c_int, _c_int, _f32p, _c_float, _c_float, _f32p]
        L.orc_xcorr_register.argtypes = [_c_int, _c_int, _f32p, _f32p, _c_int, _i64p,
                                         ctypes.POINTER(_c_int), ctypes.POINTER(_c_double)]
        L.orc_xcorr_register.restype = _c_int
        L.orc_tv_loss_grad_f64.argtypes = [_c_int, _c_int, _f32p, _f64p, _f64p, _f64p, _c_double,
                                           _c_double, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_tv_loss_grad_f64.restype = _c_double
        _lib = L
    return _lib


def _dt(prec):
    return (np.float32, "f32") if prec == 32 else (np.float64, "f64")


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def filter_taps(N, prec=32):
    dt, s = _dt(prec)
    out = np.empty(2 * N + 1, dt)
    getattr(lib(), f"orc_filter_taps_{s}")(N, out)
    return out


def cmask(N, T, wpu, prec=32):
    dt, s = _dt(prec)
    out = np.empty((N, N), dt)
    getattr(lib(), f"orc_cmask_{s}")(N, T, wpu, out)
    return out


def filter_rows(sino, prec=32):
    """tomography/tv_hpc.F90:93-105 on sino[..., T, N]."""
    dt, s = _dt(prec)
    x = _c(sino, dt)
    N, T = x.shape[-1], x.shape[-2]
    S = x.size // (N * T)
    out = np.empty_like(x)
    getattr(lib(), f"orc_filter_{s}")(N, T, S, x, out)
    return out


def backproject(sinoCS, theta, wpu, prec=32):
    dt, s = _dt(prec)
    x = _c(sinoCS, dt)
    N, T = x.shape[-1], x.shape[-2]
    S = x.size // (N * T)
    out = np.empty(x.shape[:-2] + (N, N), dt)
    getattr(lib(), f"orc_backproject_{s}")(N, T, _c(theta, np.float32), wpu, S, x, out)
    return out


def iradon(sino, theta, wpu, prec=32):
    """tomography/tv_hpc.F90:84-126 on sino[..., T, N] -> img[..., N, N]."""
    dt, s = _dt(prec)
    x = _c(sino, dt)
    N, T = x.shape[-1], x.shape[-2]
    S = x.size // (N * T)
    out = np.empty(x.shape[:-2] + (N, N), dt)
    getattr(lib(), f"orc_iradon_{s}")(N, T, _c(theta, np.float32), wpu, S, x, out)
    return out


def radon(img, theta, prec=32):
    """tomography/tv_hpc.F90:129-159 on img[..., N, N] -> sino[..., T, N]."""
    dt, s = _dt(prec)
    x = _c(img, dt)
    N = x.shape[-1]
    T = len(theta)
    S = x.size // (N * N)
    out = np.empty(x.shape[:-2] + (T, N), dt)
    getattr(lib(), f"orc_radon_{s}")(N, T, _c(theta, np.float32), S, x, out)
    return out


def radon_adjoint(sino, theta, prec=64):
    dt, s = _dt(prec)
    x = _c(sino, dt)
    N, T = x.shape[-1], x.shape[-2]
    S = x.size // (N * T)
    out = np.empty(x.shape[:-2] + (N, N), dt)
    getattr(lib(), f"orc_radon_adjoint_{s}")(N, T, _c(theta, np.float32), S, x, out)
    return out


def tvopt(f, theta, wpu, ninner, nouter, ncg, lam, mu, prec=64, red_mode=1):
    """tomography/tv_hpc.F90:162-363 on f[..., T, N]; returns (tv, fbp)."""
    dt, s = _dt(prec)
    x = _c(f, dt)
    N, T = x.shape[-1], x.shape[-2]
    S = x.size // (N * T)
    tv = np.empty(x.shape[:-2] + (N, N), dt)
    fbp = np.empty_like(tv)
    getattr(lib(), f"orc_tvopt_{s}")(N, T, _c(theta, np.float32), wpu, S, x, ninner, nouter, ncg,
                                     lam, mu, red_mode, tv, fbp.ctypes.data_as(ctypes.c_void_p))
    return tv, fbp


class CGState:
    """Work arrays of one slice's inner CG solve (tomography/tv_hpc.F90:253-300)
    for timing single CG steps: uk, r, p, Ap, irpt (N*N) and rp (T*N)."""

    def __init__(self, N, theta, wpu, lam, mu, prec=32, red_mode=0, seed=0):
        dt, self._s = _dt(prec)
        rng = np.random.default_rng(seed)
        self.N, self.theta, self.wpu = N, _c(theta, np.float32), wpu
        self.lam, self.mu, self.red = lam, mu, red_mode
        self.uk = np.zeros((N, N), dt)
        self.r = _c(rng.standard_normal((N, N)), dt)
        self.p = self.r.copy()
        self.Ap = np.empty((N, N), dt)
        self.irpt = np.empty((N, N), dt)
        self.rp = np.empty((len(theta), N), dt)
        self.rsold = float(np.sum(self.r.astype(np.float64) ** 2))

    def step(self):
        self.rsold = getattr(lib(), f"orc_cg_step_{self._s}")(
            self.N, len(self.theta), self.theta, self.wpu, self.lam, self.mu, self.red, self.uk, self.r, self.p,
            self.Ap, self.rp, self.irpt, self.rsold)
        return self.rsold


def frame_average(frames):
    x = _c(frames, np.float32)
    npix = x[0].size
    out = np.empty(x.shape[1:], np.float32)
    lib().orc_frame_average(x.shape[0], npix, x, out)
    return out


def normalize(img, ob, df, mode=0):
    x = _c(img, np.float32)
    out = np.empty_like(x)
    lib().orc_normalize(mode, x.size, x, _c(ob, np.float32), _c(df, np.float32), out)
    return out


def minloc_abs(theta, target):
    return lib().orc_minloc_abs(len(theta), _c(theta, np.float32), target)


def pick_angle(theta, proj, target):
    p = _c(proj, np.float32)
    out = np.empty(p.shape[1:], np.float32)
    lib().orc_pick_angle(len(theta), _c(theta, np.float32), p[0].size, p, target, out)
    return out


def resample(img, theta, shift):
    x = _c(img, np.float32)
    nrows, ndet = x.shape
    add = 1 if ndet % 2 == 0 else 0
    out = np.empty((nrows, ndet + add), np.float32)
    lib().orc_resample(ndet, nrows, x, theta, shift, out)
    return out


def register(p0, p180, red_mode=0):
    a, b = _c(p0, np.float32), _c(p180, np.float32)
    nrows, ndet = a.shape
    th, sh, ne = _c_float(), _c_float(), _c_int()
    lib().orc_register(ndet, nrows, a, b, red_mode, ctypes.byref(th), ctypes.byref(sh), ctypes.byref(ne))
    return th.value, sh.value, ne.value


def median27(dl, dc, dr):
    a = _c(dc, np.float32)
    nrows, ndet = a.shape
    out = np.empty_like(a)
    lib().orc_median27(ndet, nrows, _c(dl, np.float32), a, _c(dr, np.float32), out)
    return out


def proj_to_sino(proj, theta, shift):
    p = _c(proj, np.float32)
    nfiles, nrows, ndet = p.shape
    add = 1 if ndet % 2 == 0 else 0
    out = np.empty((nrows, nfiles, ndet + add), np.float32)
    lib().orc_proj_to_sino(nfiles, ndet, nrows, p, theta, shift, out)
    return out


def xcorr_register(p0, p180, kmax):
    """Returns (k_best, k_sub, corr); raises ValueError for input whose
    products are out of the fixed-point range (not finite, or >= 2^31), and
    OverflowError when a sum does not fit int64 (k_best and k_sub are then
    attached to the exception as .k_best / .k_sub)."""
    a, b = _c(p0, np.float32), _c(p180, np.float32)
    nrows, ndet = a.shape
    corr = np.empty(2 * kmax + 1, np.int64)
    kb, ks = _c_int(), _c_double()
    rc = lib().orc_xcorr_register(ndet, nrows, a, b, kmax, corr, ctypes.byref(kb), ctypes.byref(ks))
    if rc == 1:
        raise ValueError("projection value not finite, or |p0*p180| >= 2^31")
    if rc == 2:
        e = OverflowError("a correlation sum exceeds int64")
        e.k_best, e.k_sub = kb.value, ks.value
        raise e
    return kb.value, ks.value, corr


def tv_loss_grad(u, off, y, theta, lam, eps, want_grad=True):
    u = _c(u, np.float64)
    N = u.shape[-1]
    T = len(theta)
    gu = np.empty_like(u) if want_grad else None
    go = np.empty(T, np.float64) if want_grad else None
    loss = lib().orc_tv_loss_grad_f64(
        N, T, _c(theta, np.float32), u, _c(off, np.float64), _c(y, np.float64), lam, eps,
        gu.ctypes.data_as(ctypes.c_void_p) if want_grad else None,
        go.ctypes.data_as(ctypes.c_void_p) if want_grad else None)
    return (loss, gu, go) if want_grad else loss
