"""Standalone sparse matrix and Krylov solvers (mpf_sparse_*) on a caller's
reference-layout ELL matrix, against the FP64 oracle's ELL product and PCG."""
import numpy as np
import pytest

from conftest import inclusion_sigma, make_setup

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _system(alpha):
    """The FEM system S + alpha R of a 16-ring disk in the reference layout."""
    import oracle
    mesh, src, orc = make_setup(rings=16, ports=16)
    g = inclusion_sigma(mesh, seed=2)
    S = oracle.update_matrix(orc.layout, orc.layout.elemS, g, 1.0, False)
    R = oracle.update_matrix(orc.layout, orc.layout.elemR, g, 1.0, False)
    vals = oracle.update_system_matrix(orc.layout, S, R, alpha)
    return orc, vals


@pytest.mark.parametrize("solver", ["cg", "bicgstab"])
def test_sparse_solve_matches_oracle(solver):
    import oracle
    import torch
    import mpflow_gb300 as mp
    orc, vals = _system(alpha=2.5)
    n = orc.layout.n
    A = mp.SparseMatrix(vals, orc.layout.colIds, n, orc.layout.density)
    rng = np.random.default_rng(0)
    b = rng.standard_normal((n, 20))
    x_ref, _ = oracle.pcg(orc.layout, vals, b, tol=1e-14)
    x, it = A.solve(torch.tensor(b, dtype=torch.float32, device="cuda"), solver=solver, tol=1e-7)
    assert it > 0
    assert rel_err(x.cpu().numpy(), x_ref) < 1e-5
    # the product against the oracle's ELL multiply
    y = A.multiply(torch.tensor(x_ref, dtype=torch.float32, device="cuda"))
    # FP32 values and products against the FP64 oracle
    assert rel_err(y.cpu().numpy(), oracle.ell_multiply(orc.layout, vals, x_ref)) < 5e-6


def test_sparse_dc_free_and_initial_guess():
    """The singular Neumann stiffness with dcFree: (A + 1 1^T) x = b as the
    reference's iteration, from a zero and from a nonzero start."""
    import oracle
    import torch
    import mpflow_gb300 as mp
    orc, vals = _system(alpha=0.0)
    n = orc.layout.n
    A = mp.SparseMatrix(vals, orc.layout.colIds, n, orc.layout.density)
    rng = np.random.default_rng(1)
    b = rng.standard_normal((n, 3))
    b -= b.mean(axis=0)
    x_ref, _ = oracle.pcg(orc.layout, vals, b, tol=1e-14, dc_free=True)
    x, it = A.solve(torch.tensor(b, dtype=torch.float32, device="cuda"), dc_free=True, tol=1e-6)
    assert rel_err(x.cpu().numpy(), x_ref) < 1e-4
    # restarted from its own solution it needs only a few steps
    x2, it2 = A.solve(torch.tensor(b, dtype=torch.float32, device="cuda"), x0=x, dc_free=True, tol=1e-6)
    assert it2 < it // 4 and rel_err(x2.cpu().numpy(), x_ref) < 1e-4


def test_sparse_from_dense_and_errors():
    import torch
    import mpflow_gb300 as mp
    rng = np.random.default_rng(3)
    n = 300
    M = np.zeros((n, n))
    for i in range(n):
        for j in (i - 2, i - 1, i + 1, i + 2):
            if 0 <= j < n:
                M[i, j] = -rng.random()
    M = M + M.T
    M[np.arange(n), np.arange(n)] = -M.sum(axis=1) + 1.0  # SPD, diagonally dominant
    A = mp.SparseMatrix.from_dense(M)
    b = rng.standard_normal((n, 40))
    x, _ = A.solve(torch.tensor(b, dtype=torch.float32, device="cuda"), tol=1e-7)
    assert rel_err(x.cpu().numpy(), np.linalg.solve(M, b)) < 1e-5
    with pytest.raises(mp.MpfError) as e:
        A.solve(torch.tensor(b, dtype=torch.float32, device="cuda"), max_iter=1, tol=1e-12)
    assert e.value.status == 4
