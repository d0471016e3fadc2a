"""Parity at the full sizes of the 2.5D configurations: the 80-ring disk
(19441 nodes, 38400 triangles), 32 electrodes, 8 harmonics (height 4), a
seeded log-normal Gaussian random field conductivity (std 0.5, correlation
length 0.15, 4096 random Fourier features), against the FP64 oracle:
  - forward solve with FP64-residual refinement to 1e-10: voltages within
    1e-5, Jacobian (1024 x 38400) within 1e-4, reciprocity of the voltages;
  - the regularised Gauss-Newton update (split-BF16 J J^T + FP64 Cholesky)
    for four regularisation levels on 60 dB noisy data, against the oracle's
    FP64 dual solve."""
import numpy as np
import pytest

from conftest import make_setup

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def grf_conductivity(cent, seed=1, std=0.5, length=0.15, features=4096):
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((features, 2)) / length
    ph = rng.uniform(0.0, 2.0 * np.pi, features)
    field = np.sqrt(2.0 / features) * np.cos(cent @ w.T + ph).sum(axis=1)
    return np.exp(std * field / field.std())


@pytest.fixture(scope="module")
def config2():
    import oracle
    mesh, src, orc = make_setup(rings=80, ports=32, width=0.1, components=8, height=4.0)
    cent = mesh.nodes[mesh.elements].mean(axis=1)
    g = grf_conductivity(cent)
    Vo, Jo, _ = oracle.eit_forward(orc, g, tol=1e-12)
    return mesh, src, orc, g, Vo, Jo


def test_config2_forward_and_jacobian(config2):
    import torch
    import mpflow_gb300 as mp
    mesh, src, orc, g, Vo, Jo = config2
    model = mp.EIT(mesh, src, 1.0, components=8, height=4.0)
    gt = torch.tensor(g, dtype=torch.float32, device="cuda")
    V, J = model.solve(gt, mp.SolveOptions(tol=1e-6, refine_tol=1e-10, preconditioner="two-level"), jacobian=True)
    assert model.last_stats.max_rel_residual <= 1e-10
    V = V[0].cpu().numpy().astype(np.float64)
    J = J[0].cpu().numpy().astype(np.float64)
    assert V.shape == (32, 32) and J.shape == Jo.shape == (1024, 38400)
    assert rel_err(V, Vo) < 1e-5, rel_err(V, Vo)
    assert rel_err(J, Jo) < 1e-4, rel_err(J, Jo)
    # reciprocity: adjacent drive and adjacent measurement patterns are equal
    assert np.abs(V - V.T).max() <= 1e-5 * np.abs(V).max()


def test_config3_regularised_updates(config2):
    """Jacobian plus regularised inverse at the full size: J from the forward
    model, (J J^T + mu I) from split-BF16 products refined against the FP64
    normal equations, mu = (lambda_rel * rms row norm of J)^2 over four
    levels; 60 dB noisy data linearised at the homogeneous distribution."""
    import oracle
    import torch
    import mpflow_gb300 as mp
    mesh, src, orc, g, Vo, Jo = config2
    E = mesh.elements.shape[0]
    rng = np.random.default_rng(2)
    Vm = Vo + rng.standard_normal(Vo.shape) * np.sqrt((Vo ** 2).mean()) * 10 ** (-60 / 20)
    V0, J0, _ = oracle.eit_forward(orc, np.ones(E), tol=1e-12)
    y = oracle.flatten_measurement(Vm, orc) - oracle.flatten_measurement(V0, orc)
    scale = np.linalg.norm(J0) / np.sqrt(J0.shape[0])
    model = mp.EIT(mesh, src, 1.0, components=8, height=4.0)
    Vg, Jg = model.solve(torch.ones((1, E), dtype=torch.float32, device="cuda"),
                         mp.SolveOptions(tol=1e-6, refine_tol=1e-10), jacobian=True)
    vm = torch.tensor(Vm[None], dtype=torch.float32, device="cuda")  # (frames, Mm, Md) as solve() returns
    # the error split: the oracle's FP64 dual solve fed the GPU's own FP32
    # Jacobian and forward voltages isolates the solve; its distance to the
    # all-FP64 update is what the FP32 forward model contributes
    Jgd = Jg[0].cpu().numpy().astype(np.float64)
    yg = oracle.flatten_measurement(Vm, orc) - oracle.flatten_measurement(Vg[0].cpu().numpy().astype(np.float64), orc)
    errors, solve_err, model_err = {}, {}, {}
    for lam_rel in (1e-4, 1e-3, 1e-2, 1e-1):
        lam = lam_rel * scale
        want = oracle.inverse_dual(J0, y, 1.0, lam)
        want_g = oracle.inverse_dual(Jgd, yg, 1.0, lam)
        got = model.inverse(Jg[0], Vg, vm, lam, "identity")[0].cpu().numpy().astype(np.float64)
        errors[lam_rel] = rel_err(got, want)
        solve_err[lam_rel] = rel_err(got, want_g)
        model_err[lam_rel] = rel_err(want_g, want)
    print("update error vs FP64 by lambda/rms-row-norm:", errors, "solve part:", solve_err,
          "FP32 forward-model part:", model_err)
    # the solve itself (split-BF16 Gram refined in FP64) is accurate at every
    # level; the total follows the FP32 Jacobian (1e-5 relative) amplified by 1/mu
    assert all(v < 1e-3 for v in solve_err.values()), solve_err
    assert errors[1e-1] < 1e-3 and errors[1e-2] < 5e-3 and errors[1e-3] < 2e-2 and errors[1e-4] < 0.1, errors
    for lam_rel in (1e-4, 1e-3):
        assert model_err[lam_rel] > 0.5 * errors[lam_rel], (lam_rel, model_err, errors)


def test_config3_gn_step(config2):
    """One Gauss-Newton step through the batched GN path (split-BF16 Gram,
    FP64 Cholesky) at the regularisation the reconstruction bench uses."""
    import oracle
    import torch
    import mpflow_gb300 as mp
    mesh, src, orc, g, Vo, Jo = config2
    E = mesh.elements.shape[0]
    V0, J0, _ = oracle.eit_forward(orc, np.ones(E), tol=1e-12)
    y = oracle.flatten_measurement(Vo, orc) - oracle.flatten_measurement(V0, orc)
    lam = 1e-1 * np.linalg.norm(J0) / np.sqrt(J0.shape[0])
    model = mp.EIT(mesh, src, 1.0, components=8, height=4.0)
    gt = torch.ones((1, E), dtype=torch.float32, device="cuda")
    model.gn_step(gt, torch.tensor(Vo[None], dtype=torch.float32, device="cuda"), lam,
                  mp.SolveOptions(tol=1e-6, refine_tol=1e-10))
    err = rel_err(gt[0].cpu().numpy() - 1.0, oracle.inverse_dual(J0, y, 1.0, lam))
    assert err < 2e-3, err
