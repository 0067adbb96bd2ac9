"""The allocation-free prefix sum (mp_inclusive_scan_noalloc) through the C
ABI, against the library's allocating one (mp_inclusive_scan) and against
numpy's cumulative sum.

Callers such as a render loop with a fixed device-memory budget cannot let
the library call cudaMalloc/cudaFree mid-frame; this entry point takes
device buffers from the caller and keeps its scratch in a fixed __device__
array.  This file is collected last so that a failure here comes after every
other test has run; it passes alone in a fresh process and after the others.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_N = 1 << 22


def _noalloc(torch, vals):
    from micropolis_gb300 import _lib
    n = len(vals)
    din = torch.from_numpy(vals).cuda()
    dout = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    st = _lib.lib().mp_inclusive_scan_noalloc(ctypes.c_void_p(din.data_ptr()), ctypes.c_void_p(dout.data_ptr()), n,
                                              ctypes.c_void_p(stream.cuda_stream))
    assert st == _lib.MP_OK
    return dout.cpu().numpy()


def test_noalloc_scan_matches_allocating_scan(built, cuda):
    torch = cuda
    from micropolis_gb300.renderer import Renderer
    r = Renderer(window_size=(64, 64))
    rng = np.random.default_rng(11)
    # two calls in a row (the second on different, shorter data) must both be exact
    for n in (1_000_003, 4097):
        vals = rng.integers(-1000, 1000, n).astype(np.int32)
        got = _noalloc(torch, vals)
        assert np.array_equal(got, r.inclusive_scan(vals))
        assert np.array_equal(got, np.cumsum(vals, dtype=np.int64).astype(np.int32))
    r.close()


def test_noalloc_scan_at_the_limit_then_small(built, cuda):
    """n at the maximum fills every look-back tile of the scratch array; the
    small scans that follow must not see its stale tile states."""
    torch = cuda
    rng = np.random.default_rng(12)
    for n in (MAX_N, 1, 4095, 4096, 4097, 70_000):
        vals = rng.integers(-1000, 1000, n).astype(np.int32)
        assert np.array_equal(_noalloc(torch, vals), np.cumsum(vals, dtype=np.int64).astype(np.int32)), n


def test_noalloc_scan_rejects_oversize(built, cuda):
    from micropolis_gb300 import _lib
    st = _lib.lib().mp_inclusive_scan_noalloc(ctypes.c_void_p(1), ctypes.c_void_p(1), MAX_N + 1, None)
    assert st == _lib.MP_ERR_INVALID_ARG
