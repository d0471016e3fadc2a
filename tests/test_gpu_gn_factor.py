"""Factor of the Gauss-Newton system J J^T + mu I: the FP32 Cholesky (a
cluster of CTAs per frame) with FP64 iterative refinement gives the FP64
factor's update; where mu is so small that the FP32 factor breaks down or its
refinement stalls, the frame falls back to the FP64 factor and the result is
that of the FP64 path.  Reference: the regularised solve of
src/solver/inverse.cpp:213-238."""
import numpy as np
import pytest

from conftest import inclusion_sigma, make_setup

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def _problem(frames=3, rings=24):
    import torch
    import mpflow_gb300 as mp
    mesh, src, orc = make_setup(rings=rings, ports=16, logarithmic=True)
    E = mesh.elements.shape[0]
    model = mp.EIT(mesh, src, 1.0, logarithmic=True)
    vt = np.stack([10 * np.log10(inclusion_sigma(mesh, seed=s, value=v))
                   for s, v in zip(range(frames), (0.2, 5.0, 0.5, 3.0))])
    Vm = model.solve(torch.tensor(vt, dtype=torch.float32, device="cuda"),
                     mp.SolveOptions(tol=1e-7, refine_tol=1e-10))
    _, J0 = model.solve(torch.zeros((1, E), device="cuda"), mp.SolveOptions(tol=1e-7), jacobian=True)
    scale = float(J0.norm() / np.sqrt(J0.shape[1]))
    return model, Vm, E, scale, orc


def _one_update(model, Vm, E, lam, factor):
    import torch
    import mpflow_gb300 as mp
    g = torch.zeros((Vm.shape[0], E), device="cuda")
    _, _, st = model.gn_solve(g, Vm, lam, target=1e-12, max_iters=1,
                              options=mp.SolveOptions(tol=1e-7, gn_factor=factor))
    return g.cpu().numpy().astype(np.float64), st


# Both factors solve the same FP64 system to its rounding level; the update
# gamma += J^T w is then formed in FP32 from the split-BF16 J, where w (large
# at small mu) is cancelled down to gamma: one FP32 ulp of w moves gamma by
# ~1e-6 of its size, so the two updates agree to that level and no better.
@pytest.mark.parametrize("lam_rel", [0.1, 0.02])
def test_fp32_factor_matches_fp64(lam_rel):
    import oracle
    model, Vm, E, scale, orc = _problem()
    lam = lam_rel * scale
    g32, st32 = _one_update(model, Vm, E, lam, "fp32-refined")
    g64, st64 = _one_update(model, Vm, E, lam, "fp64")
    F = Vm.shape[0]
    assert st32.solves_fp32 == F and st32.solves_fp64 == 0
    assert st64.solves_fp32 == 0 and st64.solves_fp64 == F
    assert rel_err(g32, g64) < 1e-5, rel_err(g32, g64)
    # and the update is the oracle's FP64 dual step (split-BF16 Gram: ~1e-3 at these lambdas)
    V0, Jo, _ = oracle.eit_forward(orc, np.zeros(E), tol=1e-13)
    y = Vm[0].cpu().numpy().astype(np.float64).T.reshape(-1) - oracle.flatten_measurement(V0, orc)
    d_ref = oracle.inverse_dual(Jo, y, 1.0, lam)
    assert rel_err(g32[0], d_ref) < 5e-3, rel_err(g32[0], d_ref)


def test_fp32_factor_falls_back_to_fp64():
    """At lambda_rel = 1e-6 (condition ~1e12) the FP32 factor cannot solve the
    system: frames go to the FP64 factor, with the FP64 path's result."""
    model, Vm, E, scale, _ = _problem()
    lam = 1e-6 * scale
    g32, st32 = _one_update(model, Vm, E, lam, "fp32-refined")
    g64, st64 = _one_update(model, Vm, E, lam, "fp64")
    assert st32.solves_fp64 > 0, (st32.solves_fp32, st32.solves_fp64)
    assert st32.solves_fp32 + st32.solves_fp64 == Vm.shape[0]
    assert np.isfinite(g32).all()
    assert rel_err(g32, g64) < 1e-5, rel_err(g32, g64)


def test_fp32_factor_lambda_1e3_agrees_with_fp64():
    """lambda_rel = 1e-3: whichever factor solves each frame, the update is the
    FP64 path's."""
    model, Vm, E, scale, _ = _problem()
    lam = 1e-3 * scale
    g32, st32 = _one_update(model, Vm, E, lam, "fp32-refined")
    g64, _ = _one_update(model, Vm, E, lam, "fp64")
    assert st32.solves_fp32 + st32.solves_fp64 == Vm.shape[0]
    assert rel_err(g32, g64) < 1e-4, rel_err(g32, g64)
