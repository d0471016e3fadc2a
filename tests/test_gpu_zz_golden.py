"""The GPU path against the committed golden fixtures (tests/golden, made by
the FP64 oracle): the 16-ring 2D case, the 2.5D configuration reduced to 40
rings with 8 harmonics, and the complex-admittivity case.  Tolerances as the
parity tests: voltages 1e-5 with FP64 refinement (1e-4 for the FP32-only
complex solve), Jacobian 1e-4 through its products with the stored probes."""
import os

import numpy as np
import pytest

from conftest import make_setup

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def rel_err(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


@pytest.mark.parametrize("name", ["config1_small", "config2_r40"])
def test_forward_matches_golden(name):
    import torch
    import mpflow_gb300 as mp
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    extra = {"components": int(z["components"]), "height": float(z["height"])} if "components" in z.files else {}
    mesh, src, orc = make_setup(rings=int(z["rings"]), ports=int(z["ports"]), **extra)
    assert np.array_equal(orc.layout.colIds, z["colIds"]) and np.array_equal(orc.portEdges, z["portEdges"])
    model = mp.EIT(mesh, src, 1.0, **extra)
    V, J = model.solve(torch.tensor(z["sigma"], dtype=torch.float32, device="cuda")[None],
                       mp.SolveOptions(tol=1e-7, refine_tol=1e-10), jacobian=True)
    V = V[0].cpu().numpy().astype(np.float64)
    J = J[0].cpu().numpy().astype(np.float64)
    assert rel_err(V, z["V"]) < 1e-5, rel_err(V, z["V"])
    Jp = J @ z["probes"]
    assert rel_err(Jp, z["J_probe"]) < 1e-4, rel_err(Jp, z["J_probe"])


def test_complex_forward_matches_golden():
    import torch
    import mpflow_gb300 as mp
    z = np.load(os.path.join(GOLDEN, "complex_small.npz"))
    extra = {"components": int(z["components"]), "height": float(z["height"])}
    mesh, src, _ = make_setup(rings=int(z["rings"]), ports=int(z["ports"]), **extra)
    model = mp.EIT(mesh, src, 1.0, **extra)
    V, J = model.solve_complex(torch.tensor(z["gamma"][None], dtype=torch.complex64, device="cuda"),
                               mp.SolveOptions(tol=1e-7, solver="bicgstab"), jacobian=True)
    V = V[0].cpu().numpy().astype(np.complex128)
    J = J[0].cpu().numpy().astype(np.complex128)
    assert rel_err(V, z["V"]) < 1e-4, rel_err(V, z["V"])
    Jp = J @ z["probes"]
    assert rel_err(Jp, z["J_probe"]) < 1e-4, rel_err(Jp, z["J_probe"])
