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
