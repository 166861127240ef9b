"""Python mirror of the reference's Fortran module ``Tomography``
(tomography/tv_hpc.F90:1-390) on top of the C ABI.

=====================  ====================================================
reference               here
=====================  ====================================================
int_radon()             ``Tomography(nimage, theta, wpu)``  (tv_hpc.F90:11)
radon(sino, img)        ``t.radon(img)``                    (:129)
iradon(img, sino)       ``t.iradon(sino)``                  (:84)
tvopt(tv, fbp, slice)   ``t.tvopt(f, ninner, nouter, ncg, lam, mu)`` (:162)
get_slice(fbp)          ``t.get_slice(f)``                  (:365)
fin_radon()             ``t.close()``                       (:80)
=====================  ====================================================

Arrays use the Fortran storage order of the reference with the first index
fastest: ``img[..., jy-1, jx-1]``, ``sino[..., jtheta-1, jbin-1]``; leading
axes are slices.  numpy arrays go through the host-buffer entry points;
CUDA torch tensors go through the ``_dev`` entry points on torch's current
stream (float64 tensors through the ``_f64`` variants).  The module state of
the reference (ncg, nouter, lambda, mu, wpu, ...) becomes call arguments.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import call, check, lib

try:  # torch is optional for the host-buffer path
    import torch
except Exception:  # pragma: no cover
    torch = None


def _is_cuda_tensor(x):
    return torch is not None and isinstance(x, torch.Tensor) and x.is_cuda


class Tomography:
    def __init__(self, nimage: int, theta, wpu: int):
        th = np.ascontiguousarray(np.asarray(theta, dtype=np.float32))
        self.nimage = int(nimage)
        self.ntheta = int(th.size)
        self.wpu = int(wpu)
        self.theta = th
        h = ctypes.c_void_p()
        call("acu_ctx_create", ctypes.byref(h), self.nimage, self.ntheta,
             th.ctypes.data_as(ctypes.c_void_p), self.wpu)
        self._h = h

    # -- lifecycle --------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            lib().acu_ctx_destroy(self._h)
            self._h = None

    fin_radon = close

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def set_option(self, option: int, value: int):
        call("acu_set_option", self._h, int(option), int(value), ctx=self._h)

    def get_option(self, option: int) -> int:
        v = ctypes.c_int()
        call("acu_get_option", self._h, int(option), ctypes.byref(v), ctx=self._h)
        return v.value

    def _sync_stream(self):
        if torch is not None and torch.cuda.is_available():
            call("acu_set_stream", self._h, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream),
                 ctx=self._h)

    # -- helpers -------------------------------------------------------------------
    def _shape_in(self, x, kind):
        N, T = self.nimage, self.ntheta
        tail = (T, N) if kind == "sino" else (N, N)
        if tuple(x.shape[-2:]) != tail:
            raise ValueError(f"expected trailing shape {tail} ({kind}), got {tuple(x.shape)}")
        lead = tuple(x.shape[:-2])
        S = int(np.prod(lead)) if lead else 1
        return lead, S

    def _op(self, name, x, kin, kout):
        lead, S = self._shape_in(x, kin)
        N, T = self.nimage, self.ntheta
        tail = (T, N) if kout == "sino" else (N, N)
        if _is_cuda_tensor(x):
            if x.dtype == torch.float64:
                fn = name + "_dev_f64"
            elif x.dtype == torch.float32:
                fn = name + "_dev"
            else:
                raise TypeError("CUDA tensors must be float32 or float64")
            x = x.contiguous()
            out = torch.empty(lead + tail, dtype=x.dtype, device=x.device)
            self._sync_stream()
            call(fn, self._h, S, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()), ctx=self._h)
            return out
        a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
        out = np.empty(lead + tail, np.float32)
        call(name, self._h, S, a.ctypes.data_as(ctypes.c_void_p), out.ctypes.data_as(ctypes.c_void_p),
             ctx=self._h)
        return out

    # -- the module's subroutines --------------------------------------------------
    def radon(self, img):
        """tomography/tv_hpc.F90:129-159."""
        return self._op("acu_radon", img, "img", "sino")

    def iradon(self, sino):
        """tomography/tv_hpc.F90:84-126 (filter, backprojection, mask)."""
        return self._op("acu_iradon", sino, "sino", "img")

    get_slice = iradon  # tomography/tv_hpc.F90:365-386: iradon with copies

    def radon_adjoint(self, sino):
        """Exact transpose of radon (not in the reference)."""
        return self._op("acu_radon_adjoint", sino, "sino", "img")

    def filter(self, sino):
        """First half of iradon: the ramp filter (tv_hpc.F90:93-105); CUDA tensors only."""
        return self._op("acu_filter", self._cuda_only(sino), "sino", "sino")

    def backproject(self, filtered):
        """Second half of iradon (tv_hpc.F90:107-123); CUDA tensors only."""
        return self._op("acu_backproject", self._cuda_only(filtered), "sino", "img")

    @staticmethod
    def _cuda_only(x):
        if not _is_cuda_tensor(x):
            raise TypeError("filter and backproject take CUDA tensors (float32 or float64)")
        return x

    def tvopt(self, f, ninner: int, nouter: int, ncg: int, lam: float, mu: float, plain: bool = False):
        """tomography/tv_hpc.F90:162-363: returns (tv, fbp).  plain=True runs
        the per-slice reference-structured GPU path."""
        lead, S = self._shape_in(f, "sino")
        N = self.nimage
        if _is_cuda_tensor(f):
            f = f.contiguous()
            tv = torch.empty(lead + (N, N), dtype=f.dtype, device=f.device)
            fbp = torch.empty_like(tv)
            if f.dtype == torch.float64:
                if plain:
                    raise ValueError("the per-slice path is single precision")
                fn = "acu_tvopt_dev_f64"
            else:
                fn = "acu_tvopt_plain_dev" if plain else "acu_tvopt_dev"
            self._sync_stream()
            conv = float
            call(fn, self._h, S, ctypes.c_void_p(f.data_ptr()), int(ninner), int(nouter), int(ncg), conv(lam),
                 conv(mu), ctypes.c_void_p(tv.data_ptr()), ctypes.c_void_p(fbp.data_ptr()), ctx=self._h)
            return tv, fbp
        a = np.ascontiguousarray(np.asarray(f, dtype=np.float32))
        tv = np.empty(lead + (N, N), np.float32)
        fbp = np.empty_like(tv)
        call("acu_tvopt_plain" if plain else "acu_tvopt", self._h, S, a.ctypes.data_as(ctypes.c_void_p),
             int(ninner), int(nouter), int(ncg), float(lam), float(mu), tv.ctypes.data_as(ctypes.c_void_p),
             fbp.ctypes.data_as(ctypes.c_void_p), ctx=self._h)
        return tv, fbp

    # -- the batched solver in steps (device tensors) ------------------------------
    def tv_begin(self, f, ninner: int, ncg: int, lam: float, mu: float, want_fbp: bool = False):
        lead, S = self._shape_in(f, "sino")
        if not (_is_cuda_tensor(f) and f.dtype == torch.float32):
            raise TypeError("tv_begin takes a float32 CUDA tensor")
        f = f.contiguous()
        self._tv_shape = lead + (self.nimage, self.nimage)
        self._tv_keep = f
        fbp = torch.empty(self._tv_shape, dtype=f.dtype, device=f.device) if want_fbp else None
        self._sync_stream()
        call("acu_tv_begin", self._h, S, ctypes.c_void_p(f.data_ptr()), int(ninner), int(ncg), float(lam),
             float(mu), ctypes.c_void_p(fbp.data_ptr()) if want_fbp else None, ctx=self._h)
        return fbp

    def tv_iterate(self, nouter: int):
        self._sync_stream()
        call("acu_tv_iterate", self._h, int(nouter), ctx=self._h)

    def tv_end(self):
        out = torch.empty(self._tv_shape, dtype=torch.float32, device="cuda")
        self._sync_stream()
        call("acu_tv_end", self._h, ctypes.c_void_p(out.data_ptr()), ctx=self._h)
        return out

    def tv_loss_grad(self, u, off, y, lam: float, eps: float, want_grad: bool = True):
        """Registration-aware TV objective (new): returns (loss[S] float64 numpy,
        grad_u, grad_off) for CUDA tensors u[S,N,N], off[S,T] (or None),
        y[S,T,N]; float64 tensors use the double-precision kernels."""
        lead, S = self._shape_in(u, "img")
        if not (_is_cuda_tensor(u) and _is_cuda_tensor(y)):
            raise TypeError("tv_loss_grad takes CUDA tensors")
        dt = u.dtype
        u, y = u.contiguous(), y.contiguous().to(dt)
        offp = None
        if off is not None:
            off = off.contiguous().to(dt)
            offp = ctypes.c_void_p(off.data_ptr())
        gu = torch.empty_like(u) if want_grad else None
        go = torch.empty(lead + (self.ntheta,), dtype=dt, device=u.device) if (want_grad and off is not None) else None
        loss = np.zeros(S, np.float64)
        self._sync_stream()
        fn = "acu_tv_loss_grad_dev_f64" if dt == torch.float64 else "acu_tv_loss_grad_dev"
        call(fn, self._h, S, ctypes.c_void_p(u.data_ptr()), offp, ctypes.c_void_p(y.data_ptr()), float(lam),
             float(eps), loss.ctypes.data_as(ctypes.c_void_p),
             ctypes.c_void_p(gu.data_ptr()) if gu is not None else None,
             ctypes.c_void_p(go.data_ptr()) if go is not None else None, ctx=self._h)
        return loss.reshape(lead) if lead else loss[0], gu, go

    def last_delta(self, nslices: int):
        out = np.zeros(nslices, np.float64)
        call("acu_tv_last_delta", self._h, int(nslices), out.ctypes.data_as(ctypes.c_void_p), ctx=self._h)
        return out
