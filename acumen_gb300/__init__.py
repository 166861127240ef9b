"""GB300-native implementation of the Acumen tomography hot path.

The compute lives in libacumen_gpu.so (hand-written CUDA for sm_103a behind the
C ABI of include/acumen_gpu.h); this package is the host-side mirror of the
reference's Fortran ``Tomography`` module and its preprocessing programs.
"""
from ._lib import AcumenError, LIB_PATH  # noqa: F401
from . import _lib  # noqa: F401

__all__ = ["Tomography", "AcumenError", "LIB_PATH"]


def __getattr__(name):
    if name == "Tomography":
        from .tomography import Tomography
        return Tomography
    raise AttributeError(name)
