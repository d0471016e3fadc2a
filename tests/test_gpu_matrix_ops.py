"""Dense matrix operations of numeric::Matrix (mpf_matrix_*) on padded
column-major device matrices, against numpy."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(a, ld):
    """numpy (rows x cols) -> padded column-major CUDA storage (cols x ld)."""
    import torch
    rows, cols = a.shape
    buf = np.zeros((cols, ld), np.float32)
    buf[:, :rows] = a.T
    return torch.tensor(buf, device="cuda")


def _host(t, rows):
    return t.cpu().numpy()[:, :rows].T.astype(np.float64)


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def test_elementwise_and_reductions():
    import mpflow_gb300 as mp
    L = mp.lib()
    rng = np.random.default_rng(0)
    rows, cols, ld = 37, 5, 48
    A = rng.standard_normal((rows, cols))
    B = rng.standard_normal((rows, cols))
    B[3, 1] = 0.0
    dA, dB = _dev(A, ld), _dev(B, ld)
    out = _dev(np.zeros((rows, cols)), ld)
    want = {2: A + 1.5, 3: A + B, 4: 1.5 * A, 5: A * B, 6: np.where(B != 0, A / np.where(B != 0, B, 1), 0.0)}
    for op, w in want.items():
        assert L.mpf_matrix_elementwise(op, rows, cols, _p(dA), _p(dB), _p(out), ld, 1.5, None) == 0
        assert np.abs(_host(out, rows) - w).max() <= 1e-5 * np.abs(w).max(), op
    sq = _dev(A[:cols, :], 16)
    sqo = _dev(np.zeros((cols, cols)), 16)
    assert L.mpf_matrix_elementwise(1, cols, cols, _p(sq), None, _p(sqo), 16, 0.0, None) == 0
    assert np.array_equal(_host(sqo, cols), np.diag(np.diag(A[:cols, :])).astype(np.float32))
    assert L.mpf_matrix_elementwise(0, cols, cols, None, None, _p(sqo), 16, 0.0, None) == 0
    assert np.array_equal(_host(sqo, cols), np.eye(cols))
    red = {0: A.sum(axis=0), 1: (A * B).sum(axis=0), 2: A.min(axis=0), 3: A.max(axis=0)}
    for op, w in red.items():
        assert L.mpf_matrix_column_reduce(op, rows, cols, _p(dA), _p(dB), ld, _p(out), ld, None) == 0
        assert np.abs(_host(out, rows)[0] - w).max() <= 1e-5 * max(np.abs(w).max(), 1.0), op


@pytest.mark.parametrize("ta,tb", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_dense_multiply(ta, tb):
    import mpflow_gb300 as mp
    L = mp.lib()
    rng = np.random.default_rng(1)
    m, n, k = 70, 45, 130
    A = rng.standard_normal((k, m) if ta else (m, k))
    B = rng.standard_normal((n, k) if tb else (k, n))
    lda, ldb, ldc = 144, 144, 80
    dA, dB = _dev(A, lda), _dev(B, ldb)
    dC = _dev(np.zeros((m, n)), ldc)
    assert L.mpf_matrix_multiply(ta, tb, m, n, k, _p(dA), lda, _p(dB), ldb, _p(dC), ldc, None) == 0
    want = (A.T if ta else A) @ (B.T if tb else B)
    assert np.abs(_host(dC, m) - want).max() <= 1e-4 * np.abs(want).max()
