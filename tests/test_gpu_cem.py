"""Complete electrode model (contact impedance z = 1e-2 Ohm m^2 on every
electrode) on the GPU against its FP64 oracle (oracle/cem.py), at the two
configurations that specify it: 30 rings with 16 electrodes in 2D, and the
80-ring disk with 32 electrodes and 8 harmonics on a log-normal random
field.  Voltages within 1e-5 (FP64-residual refinement), Jacobian within
1e-4.  The electrode model has no counterpart in the reference, whose gap
model (src/fem/equation.cpp:183-215) the other tests cover; the two are
never compared with each other."""
import numpy as np
import pytest

from conftest import inclusion_sigma, make_setup

pytestmark = pytest.mark.gpu

Z = 1e-2


def rel_err(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def grf_conductivity(cent, seed=1, std=0.5, length=0.15, features=4096):
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((features, 2)) / length
    ph = rng.uniform(0.0, 2.0 * np.pi, features)
    field = np.sqrt(2.0 / features) * np.cos(cent @ w.T + ph).sum(axis=1)
    return np.exp(std * field / field.std())


@pytest.mark.parametrize("exact", [False, True])
def test_cem_config1_2d(exact):
    """30 rings (2791 nodes), 16 electrodes 0.1 rad wide, one harmonic,
    1 S/m with a 0.1 S/m inclusion of radius 0.2."""
    import torch
    import mpflow_gb300 as mp
    from oracle.cem import eit_forward_cem
    mesh, src, orc = make_setup(rings=30, ports=16, width=0.1, components=1)
    g = inclusion_sigma(mesh, seed=0)
    Vo, Jo, _ = eit_forward_cem(orc, g, Z, exact=exact)
    model = mp.EIT(mesh, src, 1.0, components=1, contact_impedance=Z, exact_jacobian=exact)
    assert model.info["n_nodes"] == mesh.nodes.shape[0]
    gt = torch.tensor(g, dtype=torch.float32, device="cuda")
    V, J = model.solve(gt, mp.SolveOptions(tol=1e-7, refine_tol=1e-10), jacobian=True)
    V = V[0].cpu().numpy()
    J = J[0].cpu().numpy()
    assert rel_err(V, Vo) < 1e-5, rel_err(V, Vo)
    assert rel_err(J, Jo) < 1e-4, rel_err(J, Jo)
    assert np.abs(V - V.T).max() <= 1e-5 * np.abs(V).max()


def test_cem_config2_2p5d_full_size():
    """80 rings (19441 nodes + 32 electrode voltages), 32 electrodes, 8
    harmonics (height 4), log-normal field; exact Jacobian (1024 x 38400)."""
    import torch
    import mpflow_gb300 as mp
    from oracle.cem import eit_forward_cem
    mesh, src, orc = make_setup(rings=80, ports=32, width=0.1, components=8, height=4.0)
    cent = mesh.nodes[mesh.elements].mean(axis=1)
    g = grf_conductivity(cent)
    Vo, Jo, _ = eit_forward_cem(orc, g, Z, exact=True)
    model = mp.EIT(mesh, src, 1.0, components=8, height=4.0, contact_impedance=Z, exact_jacobian=True)
    gt = torch.tensor(g, dtype=torch.float32, device="cuda")
    V, J = model.solve(gt, mp.SolveOptions(tol=1e-6, refine_tol=1e-10, preconditioner="two-level"), jacobian=True)
    assert model.last_stats.max_rel_residual <= 1e-10
    V = V[0].cpu().numpy()
    J = J[0].cpu().numpy()
    assert V.shape == (32, 32) and J.shape == Jo.shape == (1024, 38400)
    assert rel_err(V, Vo) < 1e-5, rel_err(V, Vo)
    assert rel_err(J, Jo) < 1e-4, rel_err(J, Jo)


def test_cem_gauss_newton_reaches_target():
    """Batched Gauss-Newton on the complete electrode model (log
    conductivity) reaches a 1e-3 data residual on two frames."""
    import torch
    import mpflow_gb300 as mp
    mesh, src, _ = make_setup(rings=24, ports=16, logarithmic=True)
    E = mesh.elements.shape[0]
    model = mp.EIT(mesh, src, 1.0, logarithmic=True, contact_impedance=Z)
    vt = np.stack([10 * np.log10(inclusion_sigma(mesh, seed=s, value=v)) for s, v in ((0, 0.2), (1, 5.0))])
    Vm = model.solve(torch.tensor(vt, dtype=torch.float32, device="cuda"), mp.SolveOptions(tol=1e-7, refine_tol=1e-10))
    _, J0 = model.solve(torch.zeros((1, E), device="cuda"), mp.SolveOptions(tol=1e-7), jacobian=True)
    lam = 2e-2 * float(J0.norm() / np.sqrt(J0.shape[1]))
    g = torch.zeros((2, E), device="cuda")
    iters, res, st = model.gn_solve(g, Vm, lam, target=1e-3, max_iters=10, options=mp.SolveOptions(tol=1e-6))
    assert st.frames_converged == 2 and (res <= 1e-3).all(), res
    assert (iters >= 1).all()


def test_cem_rejects_what_it_does_not_model():
    import torch
    import mpflow_gb300 as mp
    mesh, src, _ = make_setup(rings=20, ports=16)
    with pytest.raises(mp.MpfError) as e:
        mp.EIT(mesh, mp.Sources(mp.FIXED, 1.0, src.ports, src.drivePattern, src.measurementPattern), 1.0,
               contact_impedance=Z)
    assert e.value.status == 8
    model = mp.EIT(mesh, src, 1.0, contact_impedance=Z)
    with pytest.raises(mp.MpfError):
        model.solve_complex(torch.ones((1, mesh.elements.shape[0]), dtype=torch.complex64, device="cuda"))
    with pytest.raises(mp.MpfError):
        mp.EIT(mesh, src, 1.0, contact_impedance=-1.0)
