"""ctypes binding of libacumen_gpu.so (the C ABI declared in include/acumen_gpu.h).

The shared library is built in-tree by ``acumen_gb300.build.build()``.  There is
no CPU fallback: if the library is missing, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libacumen_gpu.so")

ACU_OK = 0
ACU_ERR_INVALID = -1
ACU_ERR_CUDA = -2
ACU_ERR_NOMEM = -3
ACU_ERR_TIMEOUT = -4
ACU_ERR_UNSUPPORTED = -5

ACU_OPT_FILTER = 1
ACU_OPT_LANES = 2
ACU_OPT_GRAPH = 3
ACU_OPT_VERBOSE = 4
ACU_OPT_PRINT_EVERY = 5
ACU_OPT_SLICE_BASE = 6
ACU_OPT_PROJECTOR = 7
ACU_OPT_POSITIONS = 8
ACU_OPT_RESIDUAL = 9
ACU_OPT_BP_GROUPS = 10
ACU_OPT_RADON_REFRESH = 11
ACU_OPT_BP_PARAM_TABLE = 12
ACU_OPT_MAX_BATCH = 13
ACU_OPT_BP_STAGED = 14

_ERRNAMES = {ACU_ERR_INVALID: "invalid argument", ACU_ERR_CUDA: "CUDA error", ACU_ERR_NOMEM: "out of memory",
             ACU_ERR_TIMEOUT: "device wait timed out", ACU_ERR_UNSUPPORTED: "unsupported"}


class AcumenError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_ERRNAMES.get(code, 'error')} ({code}): {msg}")
        self.code = code


_lib = None
P = ctypes.c_void_p
I = ctypes.c_int
F = ctypes.c_float
D = ctypes.c_double
L = ctypes.c_long

# name -> argument types; every function returns int
SIGNATURES = {
    "acu_ctx_create": [ctypes.POINTER(P), I, I, P, I],
    "acu_ctx_destroy": [P],
    "acu_set_stream": [P, P],
    "acu_set_option": [P, I, I],
    "acu_get_option": [P, I, ctypes.POINTER(I)],
    "acu_iradon": [P, I, P, P],
    "acu_radon": [P, I, P, P],
    "acu_radon_adjoint": [P, I, P, P],
    "acu_iradon_dev": [P, I, P, P],
    "acu_radon_dev": [P, I, P, P],
    "acu_radon_adjoint_dev": [P, I, P, P],
    "acu_filter_dev": [P, I, P, P],
    "acu_backproject_dev": [P, I, P, P],
    "acu_iradon_dev_f64": [P, I, P, P],
    "acu_radon_dev_f64": [P, I, P, P],
    "acu_radon_adjoint_dev_f64": [P, I, P, P],
    "acu_filter_dev_f64": [P, I, P, P],
    "acu_backproject_dev_f64": [P, I, P, P],
    "acu_tvopt": [P, I, P, I, I, I, F, F, P, P],
    "acu_tvopt_dev": [P, I, P, I, I, I, F, F, P, P],
    "acu_tvopt_plain": [P, I, P, I, I, I, F, F, P, P],
    "acu_tvopt_plain_dev": [P, I, P, I, I, I, F, F, P, P],
    "acu_tvopt_dev_f64": [P, I, P, I, I, I, D, D, P, P],
    "acu_tv_last_delta": [P, I, P],
    "acu_tv_begin": [P, I, P, I, I, F, F, P],
    "acu_tv_iterate": [P, I],
    "acu_tv_end": [P, P],
    "acu_frame_average_u16_dev": [P, I, L, P, P],
    "acu_frame_average_dev": [P, I, L, P, P],
    "acu_normalize_u16_dev": [P, I, I, L, P, P, P, P],
    "acu_normalize_dev": [P, I, I, L, P, P, P, P],
    "acu_pick_angle_dev": [P, I, P, L, P, F, P],
    "acu_register_dev": [P, I, I, P, P, P, P, P],
    "acu_xcorr_register_dev": [P, I, I, P, P, I, P, P, P],
    "acu_median27_dev": [P, I, I, P, P, P, P],
    "acu_resample_dev": [P, I, I, P, F, F, P],
    "acu_proj_to_sino_dev": [P, I, I, I, P, F, F, P],
    "acu_proj_to_sino_u16": [P, I, I, I, P, P, I, P, I, P, I, I, P, P, P],
    "acu_xcorr_register_noalloc": [I, I, P, P, I, P, P, P, P],
    "acu_normalize_stack_u16": [P, I, I, L, P, I, P, I, P, P],
    "acu_normalize_stack": [P, I, I, L, P, P, P, P],
    "acu_proj_to_sino": [P, I, I, I, P, P, I, P, P, P],
    "acu_tv_loss_grad_dev": [P, I, P, P, P, F, F, P, P, P],
    "acu_batch_create": [ctypes.POINTER(P), I, P, P, P, P],
    "acu_batch_destroy": [P],
    "acu_batch_set_stream": [P, P],
    "acu_batch_tvopt": [P, P, I, I, I, F, F, P, P],
    "acu_batch_op": [P, I, P, P],
    "acu_batch_tuning": [P, ctypes.POINTER(I), ctypes.POINTER(I)],
    "acu_batch_set_option": [P, I, I],
    "acu_tv_loss_grad_dev_f64": [P, I, P, P, P, D, D, P, P, P],
}


def lib():
    """Load the library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run acumen_gb300.build.build() (nvcc, sm_103a) first; "
                               "there is no CPU fallback")
        L = ctypes.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            fn = getattr(L, name, None)
            if fn is None:
                continue
            fn.argtypes = args
            fn.restype = I
        L.acu_last_error.argtypes = [P]
        L.acu_last_error.restype = ctypes.c_char_p
        if hasattr(L, "acu_batch_last_error"):
            L.acu_batch_last_error.argtypes = [P]
            L.acu_batch_last_error.restype = ctypes.c_char_p
        _lib = L
    return _lib


def check(rc: int, ctx=None):
    if rc != ACU_OK:
        msg = lib().acu_last_error(ctx)
        raise AcumenError(rc, msg.decode() if msg else "")
    return rc


def call(name: str, *args, ctx=None):
    return check(getattr(lib(), name)(*args), ctx)
