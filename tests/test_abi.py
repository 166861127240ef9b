"""CPU checks of the C ABI: the library builds, loads without a GPU, exports
every entry point include/*.h declares, and rejects bad arguments before
touching the device."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        names += re.findall(r"^\s*(?:int|const char \*|const char\*)\s*\*?\s*(acu_\w+)\s*\(", txt, re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("acu_ctx_create", "acu_iradon", "acu_radon", "acu_tvopt", "acu_radon_adjoint"):
        assert must in names


def test_library_exports_every_declared_symbol(built_lib):
    L = ctypes.CDLL(built_lib)
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing


def test_invalid_geometry_rejected_without_gpu(built_lib):
    from acumen_gb300 import _lib
    L = _lib.lib()
    h = ctypes.c_void_p()
    rc = L.acu_ctx_create(ctypes.byref(h), 2, 10, None, 4)
    assert rc == _lib.ACU_ERR_INVALID
    assert b"invalid geometry" in L.acu_last_error(None)
    rc = L.acu_ctx_create(None, 65, 10, None, 4)
    assert rc == _lib.ACU_ERR_INVALID
    assert L.acu_set_option(None, 1, 0) == _lib.ACU_ERR_INVALID


def test_python_mirror_raises_on_missing_library(tmp_path, monkeypatch):
    from acumen_gb300 import _lib
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "nope.so"))
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib.lib()


def header_constants():
    txt = "".join(open(h).read() for h in glob.glob(os.path.join(ROOT, "include", "*.h")))
    return {k: int(v) for k, v in re.findall(r"^#define\s+(ACU_(?:OPT|ERR)_\w+|ACU_OK)\s+\(?(-?\d+)\)?", txt, re.M)}


def test_binding_constants_match_the_header():
    """The option and status numbers of the Python mirror (_lib.py) and of the
    Fortran module (fortran/acumen_gpu.f90) are the header's, and each binding
    names every option the header defines."""
    from acumen_gb300 import _lib
    consts = header_constants()
    assert consts["ACU_OPT_PROJECTOR"] == 7 and consts["ACU_ERR_INVALID"] == -1
    for k, v in consts.items():
        assert getattr(_lib, k) == v, k
    f90 = open(os.path.join(ROOT, "acumen_gb300", "fortran", "acumen_gpu.f90")).read()
    fparams = {k: int(v) for k, v in re.findall(r"(ACU_\w+)\s*=\s*(-?\d+)", f90)}
    for k, v in consts.items():
        assert fparams.get(k) == v, k


def test_noalloc_registration_rejects_bad_arguments_without_gpu(built_lib):
    """acu_xcorr_register_noalloc checks its arguments before any CUDA call:
    the lag range of its fixed scratch (1..2048), the frame shape and the
    pointers.  The device pointers below are never dereferenced."""
    from acumen_gb300 import _lib
    L = _lib.lib()
    fake = ctypes.c_void_p(0x1000)
    kb, ks = ctypes.c_int(), ctypes.c_double()
    for ndet, nrows, kmax, p0, pk in ((64, 4, 0, fake, ctypes.byref(kb)), (64, 4, 2049, fake, ctypes.byref(kb)),
                                      (1, 4, 8, fake, ctypes.byref(kb)), (64, 0, 8, fake, ctypes.byref(kb)),
                                      (64, 4, 8, None, ctypes.byref(kb)), (64, 4, 8, fake, None)):
        rc = L.acu_xcorr_register_noalloc(ndet, nrows, p0, fake, kmax, None, pk, ctypes.byref(ks), None)
        assert rc == _lib.ACU_ERR_INVALID
    rc = L.acu_xcorr_register_noalloc(64, 4, fake, fake, 2049, None, ctypes.byref(kb), ctypes.byref(ks), None)
    assert b"outside 1..2048" in L.acu_last_error(None)
