"""The allocation-free registration entry point, acu_xcorr_register_noalloc.

It serves callers that cannot let the library allocate device memory (memory
reserved up front by an acquisition pipeline or owned by another allocator).
Its result must equal the context-based acu_xcorr_register_dev exactly -- the
correlation sums are integers, so "within tolerance" here means bit-exact --
on two calls in a row (the shared scratch keeps the previous call's contents
and must be cleared by each call).  The file name makes pytest collect it
last.
"""
import ctypes

import numpy as np
import pytest
import torch

from acumen_gb300 import _lib
from acumen_gb300 import synthetic as syn
from acumen_gb300.preprocess import Preprocessor

pytestmark = pytest.mark.gpu


def _pair(seed, offset):
    th, raw, flats, darks = syn.projection_stack(33, 80, 10, axis_offset=offset, seed=seed, I0=2e4)
    raw = raw.to(torch.int32).numpy().astype(np.float32)
    ob = flats.to(torch.int32).numpy().astype(np.float32).mean(0)
    p = -np.log(raw / ob)
    return (torch.from_numpy(np.ascontiguousarray(p[0])).cuda(),
            torch.from_numpy(np.ascontiguousarray(p[-1])).cuda())


def _noalloc(p0, p180, kmax):
    nrows, ndet = p0.shape
    corr = np.zeros(2 * kmax + 1, np.int64)
    kb, ks = ctypes.c_int(), ctypes.c_double()
    torch.cuda.synchronize()
    rc = _lib.lib().acu_xcorr_register_noalloc(
        ndet, nrows, ctypes.c_void_p(p0.data_ptr()), ctypes.c_void_p(p180.data_ptr()), kmax,
        corr.ctypes.data_as(ctypes.c_void_p), ctypes.byref(kb), ctypes.byref(ks),
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(rc)
    return kb.value, ks.value, corr


def test_noalloc_matches_context_entry_point_twice(built_lib):
    pp = Preprocessor()
    cases = [(_pair(3, -2.5), 16), (_pair(4, 4.0), 24)]   # two calls in a row, different lag ranges
    for (p0, p180), kmax in cases:
        kb, ks, corr = _noalloc(p0, p180, kmax)
        kr, ksr, corr_r = pp.xcorr_register(p0, p180, kmax)
        np.testing.assert_array_equal(corr, corr_r)
        assert kb == kr
        assert ks == ksr
    pp.close()


def test_noalloc_call_leaves_device_memory_unchanged(built_lib):
    """After a first call (which may load the library's device code), further
    calls allocate nothing: the device's free memory is the same before and
    after, and torch's allocator saw no new allocation."""
    p0, p180 = _pair(6, 1.5)
    _noalloc(p0, p180, 2048)                  # warm-up: the largest lag range
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    alloc0 = torch.cuda.memory_stats().get("allocation.all.allocated", 0)
    for kmax in (2048, 7):
        _noalloc(p0, p180, kmax)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert torch.cuda.memory_stats().get("allocation.all.allocated", 0) == alloc0


def test_noalloc_rejects_lag_range_beyond_scratch(built_lib):
    p0, p180 = _pair(5, 0.0)
    with pytest.raises(_lib.AcumenError, match="outside 1..2048"):
        _noalloc(p0, p180, 2049)
