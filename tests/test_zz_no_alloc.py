"""The no-allocation low-rank threshold estimate against the allocating one.

mrg_llr_update_threshold_noalloc serves callers that cannot allocate device memory
per call (a GPU memory budget reserved up front, or a pipeline that must not
synchronise the device between kernels): its scratch is a fixed array inside the
library.  This file is collected last so that a failure here leaves every other
test already run; it passes alone in a fresh process and after the others.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ip(v):
    return (ctypes.c_int * 3)(*v)


def _both(L, X, nframes, N, block, it):
    ptr = ctypes.c_void_p(X.data_ptr())
    ref, got = ctypes.c_float(), ctypes.c_float()
    assert L.mrg_llr_update_threshold(ptr, nframes, N, N, N, _ip(block), 4.0, 6.0, it, ctypes.byref(ref), None) == 0
    st = L.mrg_llr_update_threshold_noalloc(ptr, nframes, N, N, N, _ip(block), 4.0, 6.0, it, ctypes.byref(got), None)
    assert st == 0, L.mrg_last_error()
    return ref.value, got.value


def test_noalloc_matches_allocating_entry_point(mrg_lib):
    import torch
    L = mrg_lib.load()
    rng = np.random.default_rng(2024)
    for call, (nframes, N, block, it) in enumerate([(6, 32, (8, 8, 8), 0), (10, 48, (8, 8, 8), 3)]):
        X = rng.standard_normal((nframes, N, N, N)) + 1j * rng.standard_normal((nframes, N, N, N))
        Xd = torch.from_numpy(X.astype(np.complex64)).cuda()
        ref, got = _both(L, Xd, nframes, N, block, it)
        assert ref > 0
        assert abs(got - ref) <= 1e-6 * ref, (call, got, ref)
    # the result also lands in device memory when smax is a device pointer
    out = torch.zeros(1, dtype=torch.float32, device="cuda")
    assert L.mrg_llr_update_threshold_noalloc(ctypes.c_void_p(Xd.data_ptr()), 10, 48, 48, 48, _ip((8, 8, 8)), 4.0, 6.0,
                                              3, ctypes.cast(out.data_ptr(), ctypes.POINTER(ctypes.c_float)), None) == 0
    torch.cuda.synchronize()
    assert abs(float(out[0]) - ref) <= 1e-6 * ref


def test_noalloc_rejects_what_it_cannot_hold(mrg_lib):
    import torch
    L = mrg_lib.load()
    v = ctypes.c_float()
    Xh = np.zeros((2, 16, 16, 16), np.complex64)
    assert L.mrg_llr_update_threshold_noalloc(ctypes.c_void_p(Xh.ctypes.data), 2, 16, 16, 16, _ip((8, 8, 8)), 4.0,
                                              6.0, 0, ctypes.byref(v), None) == 1      # host X would need a copy
    assert b"device memory" in L.mrg_last_error()
    Xd = torch.zeros((1, 8, 8, 8), dtype=torch.complex64, device="cuda")
    # 512 x 256 x 512 voxels in 1^3 blocks is 2^26 blocks: above the fixed limit (no memory is touched)
    assert L.mrg_llr_update_threshold_noalloc(ctypes.c_void_p(Xd.data_ptr()), 1, 512, 256, 512, _ip((1, 1, 1)), 4.0,
                                              6.0, 0, ctypes.byref(v), None) == 6
    assert b"exceed the limit" in L.mrg_last_error()
    # one block past the limit: 33 x 993 x 1 blocks of one voxel = 32769
    assert L.mrg_llr_update_threshold_noalloc(ctypes.c_void_p(Xd.data_ptr()), 1, 33, 993, 1, _ip((1, 1, 1)), 4.0,
                                              6.0, 0, ctypes.byref(v), None) == 6
    # 2^16 x 2^16 x 2^16 blocks: 2^48, which a 32-bit count would have wrapped to 0
    assert L.mrg_llr_update_threshold_noalloc(ctypes.c_void_p(Xd.data_ptr()), 1, 65536, 65536, 65536,
                                              _ip((1, 1, 1)), 4.0, 6.0, 0, ctypes.byref(v), None) == 6
    # a block edge below 1
    assert L.mrg_llr_update_threshold_noalloc(ctypes.c_void_p(Xd.data_ptr()), 1, 8, 8, 8, _ip((0, 8, 8)), 4.0,
                                              6.0, 0, ctypes.byref(v), None) == 1


def test_noalloc_at_the_limit_then_smaller(mrg_lib):
    """Exactly MRG_NOALLOC_MAX_BLOCKS blocks (64^3 in 2^3 blocks, 2 frames) fill the sort
    buffer to its end; a smaller call right after must not see the larger call's leftovers."""
    import torch
    L = mrg_lib.load()
    rng = np.random.default_rng(77)
    for nframes, N, block, it in [(2, 64, (2, 2, 2), 1), (6, 32, (8, 8, 8), 0), (2, 64, (2, 2, 2), 5)]:
        X = rng.standard_normal((nframes, N, N, N)) + 1j * rng.standard_normal((nframes, N, N, N))
        Xd = torch.from_numpy(X.astype(np.complex64)).cuda()
        ref, got = _both(L, Xd, nframes, N, block, it)
        assert ref > 0
        assert abs(got - ref) <= 1e-6 * ref, (nframes, N, block, got, ref)
