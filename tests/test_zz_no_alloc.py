"""The allocation-free normalisation entry point, through the C ABI.

It is meant for callers that must not have a library allocate device memory
(a reconstruction loop holding a fixed, pre-reserved memory budget, or a host
application whose allocator owns the device), so it takes no context and
keeps its scratch in a fixed array inside libfbp.  This file is collected
last: the entry point's state outlives every call, and the checks below must
hold both in a fresh process and after every other test has run.
"""
import ctypes

import pytest
import torch

pytestmark = pytest.mark.gpu


def _noalloc(lib, t, stream):
    return lib.fbp_normalize_minmax_noalloc(ctypes.c_void_p(t.data_ptr()), t.numel(), ctypes.c_void_p(stream))


def test_noalloc_matches_context_entry_point_twice(built, cuda):
    from fasterbackprojection_gb300 import _lib
    from fasterbackprojection_gb300.api import Context

    lib = _lib.load()
    stream = torch.cuda.current_stream().cuda_stream
    g = torch.Generator(device="cpu").manual_seed(123)
    with Context(0) as ctx:
        # Two calls in a row, different sizes: the second must not see the first's scratch.
        for n in (3_000_001, 77_777):
            x = (torch.randn(n, generator=g) * 5 + 1).to(cuda)
            want = ctx.normalize_(x.clone())
            got = x.clone()
            assert _noalloc(lib, got, stream) == _lib.FBP_OK, lib.fbp_last_error()
            torch.cuda.synchronize()
            assert torch.equal(got, want)
            assert float(got.min()) == 0.0 and float(got.max()) == 1.0


def test_noalloc_rejects_oversized_input(built, cuda):
    from fasterbackprojection_gb300 import _lib

    lib = _lib.load()
    x = torch.zeros(16, device=cuda)
    st = lib.fbp_normalize_minmax_noalloc(ctypes.c_void_p(x.data_ptr()), (1 << 30) + 1, None)
    assert st == _lib.FBP_ERR_UNSUPPORTED
    assert b"2^30" in lib.fbp_last_error()
    assert lib.fbp_normalize_minmax_noalloc(None, 16, None) == _lib.FBP_ERR_INVALID_ARG


def test_noalloc_rejects_host_memory(built, cuda):
    from fasterbackprojection_gb300 import _lib

    lib = _lib.load()
    host = (ctypes.c_float * 64)()
    st = lib.fbp_normalize_minmax_noalloc(ctypes.cast(host, ctypes.c_void_p), 64, None)
    assert st == _lib.FBP_ERR_INVALID_ARG
    assert b"device memory" in lib.fbp_last_error()
