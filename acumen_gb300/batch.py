"""Ragged batches of independent problems (different grid side and angle count),
solved together by the C ABI's acu_batch_* entry points (persistent kernels
over (problem, angle, bin block) / (problem, pixel tile) work lists)."""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import AcumenError, call, lib


class RaggedBatch:
    def __init__(self, nimage, thetas, wpu):
        self.N = [int(n) for n in nimage]
        self.thetas = [np.ascontiguousarray(np.asarray(t, np.float32)) for t in thetas]
        self.T = [len(t) for t in self.thetas]
        wp = [int(wpu)] * len(self.N) if np.isscalar(wpu) else [int(w) for w in wpu]
        n = len(self.N)
        ni = (ctypes.c_int * n)(*self.N)
        nt = (ctypes.c_int * n)(*self.T)
        nw = (ctypes.c_int * n)(*wp)
        th = np.ascontiguousarray(np.concatenate(self.thetas))
        h = ctypes.c_void_p()
        call("acu_batch_create", ctypes.byref(h), n, ni, nt, th.ctypes.data_as(ctypes.c_void_p), nw)
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().acu_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise AcumenError(rc, lib().acu_batch_last_error(self._h).decode())

    def _pack(self, arrs, shapes):
        out = []
        for a, s in zip(arrs, shapes):
            a = np.ascontiguousarray(np.asarray(a, np.float32))
            if a.shape != s:
                raise ValueError(f"expected {s}, got {a.shape}")
            out.append(a.ravel())
        return np.ascontiguousarray(np.concatenate(out))

    def _unpack(self, flat, shapes):
        res, o = [], 0
        for s in shapes:
            n = int(np.prod(s))
            res.append(flat[o:o + n].reshape(s))
            o += n
        return res

    def tvopt(self, sinos, ninner, nouter, ncg, lam, mu):
        ss = [(t, n) for n, t in zip(self.N, self.T)]
        si = [(n, n) for n in self.N]
        f = self._pack(sinos, ss)
        tot = sum(n * n for n in self.N)
        tv = np.empty(tot, np.float32)
        fbp = np.empty(tot, np.float32)
        self._check(lib().acu_batch_tvopt(self._h, f.ctypes.data_as(ctypes.c_void_p), ninner, nouter, ncg, lam, mu,
                                          tv.ctypes.data_as(ctypes.c_void_p), fbp.ctypes.data_as(ctypes.c_void_p)))
        return self._unpack(tv, si), self._unpack(fbp, si)

    def radon(self, imgs):
        si = [(n, n) for n in self.N]
        ss = [(t, n) for n, t in zip(self.N, self.T)]
        x = self._pack(imgs, si)
        out = np.empty(sum(t * n for n, t in zip(self.N, self.T)), np.float32)
        self._check(lib().acu_batch_op(self._h, 0, x.ctypes.data_as(ctypes.c_void_p), out.ctypes.data_as(ctypes.c_void_p)))
        return self._unpack(out, ss)

    def iradon(self, sinos):
        si = [(n, n) for n in self.N]
        ss = [(t, n) for n, t in zip(self.N, self.T)]
        x = self._pack(sinos, ss)
        out = np.empty(sum(n * n for n in self.N), np.float32)
        self._check(lib().acu_batch_op(self._h, 1, x.ctypes.data_as(ctypes.c_void_p), out.ctypes.data_as(ctypes.c_void_p)))
        return self._unpack(out, si)

    def tuning(self):
        w, r = ctypes.c_int(), ctypes.c_int()
        self._check(lib().acu_batch_tuning(self._h, ctypes.byref(w), ctypes.byref(r)))
        return w.value, r.value

    def set_option(self, option, value):
        """acu_batch_set_option: ACU_OPT_POSITIONS (8) and ACU_OPT_RADON_REFRESH (11)."""
        self._check(lib().acu_batch_set_option(self._h, int(option), int(value)))
