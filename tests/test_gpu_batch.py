"""Batches of uneven meshes (mpf_batch_*): the voltages every model gets from
the shared CG launches equal its own forward solve and the FP64 oracle."""
import numpy as np
import pytest

from conftest import inclusion_sigma, make_setup

pytestmark = pytest.mark.gpu

# (rings, electrodes, port width in rad): unique excitations 16, 32, 8 ->
# width classes 16 and 32; every port spans at least one boundary edge
CASES = [(12, 16, 0.2), (14, 32, 0.17), (10, 8, 0.3), (18, 16, 0.2), (9, 16, 0.3)]
FRAMES = 3


def rel_err(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _setups(components=4, height=4.0, cases=CASES):
    import mpflow_gb300 as mp
    out = []
    for rings, ports, width in cases:
        mesh, src, orc = make_setup(rings=rings, ports=ports, width=width, components=components, height=height)
        model = mp.EIT(mesh, src, 1.0, components=components, height=height)
        out.append((mesh, orc, model))
    return out


def _frames(mesh, seed):
    """A circular inclusion moving over FRAMES frames (contrast 0.2, radius 0.25)."""
    cent = mesh.nodes[mesh.elements].mean(axis=1)
    g = np.ones((FRAMES, mesh.elements.shape[0]))
    for f in range(FRAMES):
        t = 2 * np.pi * (seed + f) / 7.0
        c = 0.45 * np.array([np.cos(t), np.sin(t)])
        g[f, np.linalg.norm(cent - c, axis=1) < 0.25] = 0.2
    return g


def test_batch_matches_single_models_and_oracle():
    import oracle
    import torch
    import mpflow_gb300 as mp
    setups = _setups()
    gammas = [torch.tensor(_frames(mesh, i), dtype=torch.float32, device="cuda") for i, (mesh, _, _) in
              enumerate(setups)]
    batch = mp.EITBatch([m for _, _, m in setups])
    opts = mp.SolveOptions(tol=1e-7)
    Vb = batch.solve(gammas, opts)
    assert batch.last_stats.not_converged == 0
    # two width classes, three launch shapes each
    assert batch.cg_variants(FRAMES).shape == (2, 3)
    for i, (mesh, orc, model) in enumerate(setups):
        Vs = model.solve(gammas[i], opts)
        assert Vb[i].shape == Vs.shape
        assert rel_err(Vb[i].cpu().numpy(), Vs.cpu().numpy()) < 2e-5, i
    # FP64 oracle for the smallest and the largest mesh (frame 1)
    for i in (4, 3):
        mesh, orc, _ = setups[i]
        Vo, _, _ = oracle.eit_forward(orc, _frames(mesh, i)[1], tol=1e-13, want_jacobian=False)
        assert rel_err(Vb[i][1].cpu().numpy(), Vo) < 1e-4, i
    # per-system convergence masks: each group stops on its own
    it = batch.iterations(FRAMES)
    assert it.shape == (len(CASES), FRAMES, 4)
    assert (it > 0).all()
    assert it[4].max() < it[3].max()  # 9 rings stop before 18 rings
    ms, by = batch.cg_stats()
    assert ms > 0 and by > 0


def test_batch_two_level_matches_single_models():
    """Every mesh of the batch gets its own coarse space (padded to the
    largest of its width class): same voltages, fewer iterations."""
    import oracle
    import torch
    import mpflow_gb300 as mp
    setups = _setups()
    gammas = [torch.tensor(_frames(mesh, i), dtype=torch.float32, device="cuda") for i, (mesh, _, _) in
              enumerate(setups)]
    batch = mp.EITBatch([m for _, _, m in setups])
    jac = mp.SolveOptions(tol=1e-7)
    two = mp.SolveOptions(tol=1e-7, preconditioner="two-level")
    Vj = batch.solve(gammas, jac)
    it_j = batch.iterations(FRAMES)
    Vt = batch.solve(gammas, two)
    it_t = batch.iterations(FRAMES)
    assert batch.last_stats.not_converged == 0
    for i, (mesh, orc, model) in enumerate(setups):
        Vs = model.solve(gammas[i], two)
        assert rel_err(Vt[i].cpu().numpy(), Vs.cpu().numpy()) < 2e-5, i
        assert rel_err(Vt[i].cpu().numpy(), Vj[i].cpu().numpy()) < 2e-5, i
    mesh, orc, _ = setups[3]
    Vo, _, _ = oracle.eit_forward(orc, _frames(mesh, 3)[0], tol=1e-13, want_jacobian=False)
    assert rel_err(Vt[3][0].cpu().numpy(), Vo) < 1e-4
    # the largest mesh needs fewer iterations with its coarse space
    assert it_t[3].max() < it_j[3].max()


# SpMM codes 72..143 are the tile-staged form (bulk copies of each tile's own
# and halo rows, 2 or 3 stages) over the stacked meshes' tiles
@pytest.mark.parametrize("shapes", [[1, 13, 22], [28, 4, 8], [35, 31, 10], [100, 13, 22], [108, 4, 8],
                                    [130, 31, 10]])
def test_batch_forced_launch_shapes(shapes):
    import torch
    import mpflow_gb300 as mp
    setups = _setups(cases=CASES[:3])
    gammas = [torch.tensor(_frames(mesh, i), dtype=torch.float32, device="cuda") for i, (mesh, _, _) in
              enumerate(setups)]
    batch = mp.EITBatch([m for _, _, m in setups])
    opts = mp.SolveOptions(tol=1e-7)
    ref = batch.solve(gammas, opts)
    got = batch.cg_variants(FRAMES, set=shapes)
    assert (got == np.array(shapes)).all()
    V = batch.solve(gammas, opts)
    for a, b in zip(V, ref):
        assert rel_err(a.cpu().numpy(), b.cpu().numpy()) < 2e-5


def test_batch_rejects_other_harmonic_sets():
    import mpflow_gb300 as mp
    a = _setups(components=4, cases=CASES[:1])[0][2]
    b = _setups(components=2, cases=CASES[:1])[0][2]
    with pytest.raises(mp.MpfError) as e:
        mp.EITBatch([a, b])
    assert e.value.status == 1


def test_batch_rejects_refinement_and_warm_start():
    import torch
    import mpflow_gb300 as mp
    (mesh, _, model), = _setups(cases=CASES[:1])
    batch = mp.EITBatch([model])
    g = [torch.ones((1, mesh.elements.shape[0]), dtype=torch.float32, device="cuda")]
    for opts in (mp.SolveOptions(refine_tol=1e-10), mp.SolveOptions(warm_start=True)):
        with pytest.raises(mp.MpfError) as e:
            batch.solve(g, opts)
        assert e.value.status == 8


def test_batch_config4_largest_members_full_size():
    """Configuration 4's largest members at full size in one batch: the
    100-ring disk (30301 nodes) with 16 and with 32 electrodes, 4 harmonics
    (height 4), beside a 20-ring one; every mesh's voltages against the FP64
    oracle (the per-mesh solve of src/models/eit.cpp:139-213)."""
    import oracle
    import torch
    import mpflow_gb300 as mp
    cases = [(100, 16, 0.1), (100, 32, 0.1), (20, 16, 0.1)]
    setups = _setups(cases=cases)
    gammas = [torch.tensor(_frames(mesh, i)[:2], dtype=torch.float32, device="cuda")
              for i, (mesh, _, _) in enumerate(setups)]
    batch = mp.EITBatch([m for _, _, m in setups])
    Vb = batch.solve(gammas, mp.SolveOptions(tol=1e-6, preconditioner="two-level"))
    assert batch.last_stats.not_converged == 0
    for i, (mesh, orc, _) in enumerate(setups):
        Vo, _, _ = oracle.eit_forward(orc, _frames(mesh, i)[1], tol=1e-12, want_jacobian=False)
        assert rel_err(Vb[i][1].cpu().numpy(), Vo) < 1e-4, (i, rel_err(Vb[i][1].cpu().numpy(), Vo))
