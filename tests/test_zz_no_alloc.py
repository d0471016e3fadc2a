"""The allocation-free Gram entry point (mpf_gram_split_bf16_noalloc).

It exists for callers that cannot allocate device memory once running (a
real-time loop that must not stall on cudaMalloc's device synchronisation, or
a host framework whose allocator owns the device): its scratch lives in fixed
device arrays inside the library.  This file is collected last on purpose, so
that a failure here does not hide the results of the other tests; it passes
both alone in a fresh process and after the rest of the suite.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call_noalloc(A, C):
    import torch
    from mpflow_gb300._ffi import lib, ptr
    B, rows, cols = A.shape
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    return lib().mpf_gram_split_bf16_noalloc(B, rows, cols, ptr(A), cols, ptr(C), stream)


def test_noalloc_gram_matches_allocating_entry_point_twice():
    import torch
    import mpflow_gb300 as mp
    rng = np.random.default_rng(11)
    for call in range(2):
        A = torch.tensor(rng.standard_normal((2, 256, 640)).astype(np.float32), device="cuda")
        expected = mp.gram_split_bf16(A)
        C = torch.full((2, 256, 256), float("nan"), dtype=torch.float32, device="cuda")
        assert _call_noalloc(A, C) == 0, mp.lib().mpf_last_error()
        got = C.cpu().numpy()
        ref = expected.cpu().numpy()
        # same kernels and split rule: agreement within the Gram test's 3e-5 tolerance
        err = np.abs(got - ref).max() / np.abs(ref).max()
        assert err < 3e-5, (call, err)
        # and against FP64 directly
        Ad = A.cpu().numpy().astype(np.float64)
        exact = np.einsum("bik,bjk->bij", Ad, Ad)
        assert np.abs(got - exact).max() / np.abs(exact).max() < 3e-5


def test_noalloc_gram_rejects_requests_beyond_its_scratch():
    import torch
    import mpflow_gb300 as mp
    A = torch.zeros((1, 1024, 4096), dtype=torch.float32, device="cuda")  # 4 Mi elements > 2 Mi
    C = torch.zeros((1, 1024, 1024), dtype=torch.float32, device="cuda")
    assert _call_noalloc(A, C) == 1  # MPF_EINVAL
    assert b"exceeds the fixed scratch" in mp.lib().mpf_last_error()
