"""Failure detection on the GPU without a fault: a bounded device wait that
nothing satisfies gives up after its limit, the call returns MPF_ETIMEOUT
and the context stays usable."""
import time

import numpy as np
import pytest

from conftest import make_setup

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_context_survives():
    import torch
    import mpflow_gb300 as mp
    L = mp.lib()
    t0 = time.perf_counter()
    status = L.mpf_selftest_bounded_wait(50000, None)  # 50 ms
    elapsed = time.perf_counter() - t0
    assert status == 6, L.mpf_last_error()
    assert b"bounded wait ran out" in L.mpf_last_error()
    assert elapsed < 5.0
    # the same context runs a forward solve afterwards
    mesh, src, _ = make_setup(rings=12, ports=16, width=0.2)
    model = mp.EIT(mesh, src, 1.0)
    V = model.solve(torch.ones((1, mesh.elements.shape[0]), device="cuda"), mp.SolveOptions(tol=1e-6))
    assert torch.isfinite(V).all() and float(V.abs().max()) > 0
    assert model.last_stats.not_converged == 0


def test_gn_solve_freezes_a_diverging_frame():
    """A frame whose Gauss-Newton update leaves the forward model's range
    (here: non-finite measurements, so a non-finite step) is undone and
    frozen unconverged; the other frames of the batch still converge."""
    import torch
    import mpflow_gb300 as mp
    from mpflow_gb300.learned import inclusion_frames
    mesh, src, _ = make_setup(rings=20, ports=16, logarithmic=True)
    E = mesh.elements.shape[0]
    model = mp.EIT(mesh, src, 1.0, logarithmic=True)
    cent = mesh.nodes[mesh.elements].mean(axis=1)
    g_true = inclusion_frames(cent, 4, np.random.default_rng(3))
    V = model.solve(torch.tensor(g_true, device="cuda"), mp.SolveOptions(tol=1e-6, refine_tol=1e-10)).contiguous()
    V[2, 0, 0] = float("nan")
    _, J0 = model.solve(torch.zeros((1, E), device="cuda"), mp.SolveOptions(tol=1e-6), jacobian=True)
    lam = 2e-2 * float(J0.norm() / np.sqrt(J0.shape[1]))
    g = torch.zeros((4, E), device="cuda")
    it, res, st = model.gn_solve(g, V, lam, target=1e-3, max_iters=8, options=mp.SolveOptions(tol=1e-6))
    assert st.frames_converged == 3
    assert all(res[f] <= 1e-3 for f in (0, 1, 3)), res
    assert it[2] == 1 and bool(torch.isfinite(g).all())
    assert float(g[2].abs().max()) == 0.0  # the undone update left the start
