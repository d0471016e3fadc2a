"""Batched BiCGSTAB (mpf_solve_opts.solver = 1) against the FP64 oracle's
restatement of BiCGSTAB::solve and against the CG path, through the C ABI."""
import numpy as np
import pytest

from conftest import inclusion_sigma, make_setup

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("refine", [0.0, 1e-10])
def test_bicgstab_forward_matches_oracle(refine):
    import oracle
    import torch
    import mpflow_gb300 as mp
    mesh, src, orc = make_setup(rings=16, ports=32, width=0.1, components=4, height=4.0)
    rng = np.random.default_rng(4)
    g = np.exp(0.3 * rng.standard_normal(mesh.elements.shape[0]))
    Vo, Jo, _ = oracle.eit_forward(orc, g, tol=1e-13, solver="bicgstab")
    model = mp.EIT(mesh, src, 1.0, components=4, height=4.0)
    gt = torch.tensor(g, dtype=torch.float32, device="cuda")
    V, J = model.solve(gt, mp.SolveOptions(tol=1e-7, refine_tol=refine, solver="bicgstab"), jacobian=True)
    assert model.last_stats.not_converged == 0 and model.last_stats.iterations > 0
    tolV = 1e-5 if refine else 1e-4
    assert rel_err(V[0].cpu().numpy(), Vo) < tolV
    assert rel_err(J[0].cpu().numpy(), Jo) < 1e-4


def test_bicgstab_fields_match_cg_and_need_fewer_iterations():
    import torch
    import mpflow_gb300 as mp
    mesh, src, _ = make_setup(rings=24, ports=16, components=3, height=2.0)
    g = torch.tensor(np.stack([inclusion_sigma(mesh, seed=s) for s in range(3)]), dtype=torch.float32,
                     device="cuda")
    model = mp.EIT(mesh, src, 1.0, components=3, height=2.0)
    Vc = model.solve(g, mp.SolveOptions(tol=1e-7))
    Fc = model.fields(3).cpu().numpy()
    it_cg = model.group_iterations()
    Vb = model.solve(g, mp.SolveOptions(tol=1e-7, solver="bicgstab"))
    Fb = model.fields(3).cpu().numpy()
    it_bi = model.group_iterations()
    assert rel_err(Vb.cpu().numpy(), Vc.cpu().numpy()) < 2e-5
    n = mesh.nodes.shape[0]
    # same system (A + c' 1 1^T on the Neumann harmonic), same fields
    assert rel_err(Fb[..., :n], Fc[..., :n]) < 2e-5
    # two SpMVs per BiCGSTAB iteration, fewer iterations than CG
    assert it_bi.max() < it_cg.max()


def test_bicgstab_warm_start_and_batch():
    import torch
    import mpflow_gb300 as mp
    cases = [(12, 16, 0.2), (18, 16, 0.2), (14, 32, 0.17)]
    models, gammas = [], []
    for i, (rings, ports, width) in enumerate(cases):
        mesh, src, _ = make_setup(rings=rings, ports=ports, width=width, components=3, height=2.0)
        models.append(mp.EIT(mesh, src, 1.0, components=3, height=2.0))
        gammas.append(torch.tensor(np.stack([inclusion_sigma(mesh, seed=10 * i + f) for f in range(2)]),
                                   dtype=torch.float32, device="cuda"))
    cg = mp.SolveOptions(tol=1e-7)
    bi = mp.SolveOptions(tol=1e-7, solver="bicgstab")
    batch = mp.EITBatch(models)
    Vb = batch.solve(gammas, bi)
    assert batch.last_stats.not_converged == 0
    for m, g, v in zip(models, gammas, Vb):
        Vs = m.solve(g, cg)
        assert rel_err(v.cpu().numpy(), Vs.cpu().numpy()) < 2e-5
        # warm start from the fields just computed: converges at once
        Vw = m.solve(g, mp.SolveOptions(tol=1e-6, solver="bicgstab", warm_start=True))
        assert rel_err(Vw.cpu().numpy(), Vs.cpu().numpy()) < 2e-5
        assert m.group_iterations().max() <= 2
    ms, by = batch.cg_stats()
    assert ms > 0 and by > 0
