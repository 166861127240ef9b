"""Host-side mirror of the reference's projection-preprocessing programs on the
C ABI: tomography/fits_to_hpc.F90 (flat/dark averages and log-normalisation)
and tomography/projections_to_sinogram_hpc.F90 (0/180-degree projections,
rotation-axis registration, 27-point median, resample, transpose to slice-major
sinograms).

Images are ``[..., nrows, ndet]`` arrays (detector fastest).  The functions
take CUDA torch tensors and run on torch's current stream; ``proj_to_sino_u16``
also accepts host numpy arrays and runs the whole chain.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from ._lib import call, lib


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class Preprocessor:
    """A library context without a reconstruction grid (nimage = 0)."""

    def __init__(self):
        h = ctypes.c_void_p()
        call("acu_ctx_create", ctypes.byref(h), 0, 0, None, 0)
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().acu_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _stream(self):
        call("acu_set_stream", self._h, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), ctx=self._h)

    # fits_to_hpc.F90:183-210
    def frame_average(self, frames):
        frames = frames.contiguous()
        out = torch.empty(frames.shape[1:], dtype=torch.float32, device=frames.device)
        npix = out.numel()
        self._stream()
        if frames.dtype == torch.float32:
            call("acu_frame_average_dev", self._h, frames.shape[0], npix, _ptr(frames), _ptr(out), ctx=self._h)
        else:
            call("acu_frame_average_u16_dev", self._h, frames.shape[0], npix, _ptr(frames), _ptr(out), ctx=self._h)
        return out

    # fits_to_hpc.F90:243 (mode 0) / :244 (mode 1)
    def normalize(self, raw, ob, df=None, mode=0):
        raw = raw.contiguous()
        npix = ob.numel()
        nproj = raw.numel() // npix
        out = torch.empty(raw.shape, dtype=torch.float32, device=raw.device)
        dfp = _ptr(df.contiguous()) if df is not None else None
        self._stream()
        name = "acu_normalize_dev" if raw.dtype == torch.float32 else "acu_normalize_u16_dev"
        call(name, self._h, int(mode), nproj, npix, _ptr(raw), _ptr(ob.contiguous()), dfp, _ptr(out), ctx=self._h)
        return out

    # projections_to_sinogram_hpc.F90:141-224
    def pick_angle(self, theta, proj, target):
        th = np.ascontiguousarray(np.asarray(theta, np.float32))
        proj = proj.contiguous()
        out = torch.empty(proj.shape[1:], dtype=torch.float32, device=proj.device)
        self._stream()
        call("acu_pick_angle_dev", self._h, len(th), th.ctypes.data_as(ctypes.c_void_p), out.numel(), _ptr(proj),
             float(target), _ptr(out), ctx=self._h)
        return out

    # :231-364
    def register(self, p0, p180):
        nrows, ndet = p0.shape
        th, sh, ne = ctypes.c_float(), ctypes.c_float(), ctypes.c_int()
        self._stream()
        call("acu_register_dev", self._h, ndet, nrows, _ptr(p0.contiguous()), _ptr(p180.contiguous()),
             ctypes.byref(th), ctypes.byref(sh), ctypes.byref(ne), ctx=self._h)
        return th.value, sh.value, ne.value

    def xcorr_register(self, p0, p180, kmax, want_corr=True):
        """(k_best, k_sub, corr); corr is None with want_corr=False, which also
        serves sums beyond the int64 range of corr_out."""
        nrows, ndet = p0.shape
        corr = np.zeros(2 * kmax + 1, np.int64) if want_corr else None
        kb, ks = ctypes.c_int(), ctypes.c_double()
        self._stream()
        call("acu_xcorr_register_dev", self._h, ndet, nrows, _ptr(p0.contiguous()), _ptr(p180.contiguous()),
             int(kmax), corr.ctypes.data_as(ctypes.c_void_p) if want_corr else None, ctypes.byref(kb),
             ctypes.byref(ks), ctx=self._h)
        return kb.value, ks.value, corr

    # :426-452
    def median27(self, dl, dc, dr):
        nrows, ndet = dc.shape
        out = torch.empty_like(dc)
        self._stream()
        call("acu_median27_dev", self._h, ndet, nrows, _ptr(dl.contiguous()), _ptr(dc.contiguous()),
             _ptr(dr.contiguous()), _ptr(out), ctx=self._h)
        return out

    # :456-470
    def resample(self, img, theta, shift):
        nrows, ndet = img.shape
        add = 1 if ndet % 2 == 0 else 0
        out = torch.empty(nrows, ndet + add, dtype=torch.float32, device=img.device)
        self._stream()
        call("acu_resample_dev", self._h, ndet, nrows, _ptr(img.contiguous()), float(theta), float(shift),
             _ptr(out), ctx=self._h)
        return out

    # :397-487
    def proj_to_sino(self, proj, theta, shift):
        nproj, nrows, ndet = proj.shape
        add = 1 if ndet % 2 == 0 else 0
        out = torch.empty(nrows, nproj, ndet + add, dtype=torch.float32, device=proj.device)
        self._stream()
        call("acu_proj_to_sino_dev", self._h, nproj, ndet, nrows, _ptr(proj.contiguous()), float(theta),
             float(shift), _ptr(out), ctx=self._h)
        return out

    def proj_to_sino_u16(self, raw, theta, flats, darks=None, norm_mode=0, reg_method=0):
        """The whole chain on host arrays; returns (sinograms, theta, shift)."""
        raw = np.ascontiguousarray(raw, np.uint16)
        flats = np.ascontiguousarray(flats, np.uint16)
        th = np.ascontiguousarray(np.asarray(theta, np.float32))
        nproj, nrows, ndet = raw.shape
        add = 1 if ndet % 2 == 0 else 0
        out = np.empty((nrows, nproj, ndet + add), np.float32)
        if darks is not None:
            darks = np.ascontiguousarray(darks, np.uint16)
        t_out, s_out = ctypes.c_float(), ctypes.c_float()
        call("acu_proj_to_sino_u16", self._h, nproj, ndet, nrows, raw.ctypes.data_as(ctypes.c_void_p),
             th.ctypes.data_as(ctypes.c_void_p), flats.shape[0], flats.ctypes.data_as(ctypes.c_void_p),
             0 if darks is None else darks.shape[0],
             None if darks is None else darks.ctypes.data_as(ctypes.c_void_p), int(norm_mode), int(reg_method),
             out.ctypes.data_as(ctypes.c_void_p), ctypes.byref(t_out), ctypes.byref(s_out), ctx=self._h)
        return out, t_out.value, s_out.value
