"""GPU parity of the CUDA path against the FP64 oracle, through the C ABI."""
import numpy as np
import pytest

from conftest import inclusion_sigma, make_setup

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    return torch


def rel_err(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def test_assembly_matches_oracle():
    import oracle
    import mpflow_gb300 as mp
    torch = _torch()
    mesh, src, orc = make_setup(rings=16)
    g = inclusion_sigma(mesh, seed=3)
    model = mp.EIT(mesh, src, 1.0)
    S, R = model.assemble(torch.tensor(g, dtype=torch.float32, device="cuda"))
    S, R = S[0].cpu().numpy(), R[0].cpu().numpy()
    So = oracle.update_matrix(orc.layout, orc.layout.elemS, g, 1.0, False)
    Ro = oracle.update_matrix(orc.layout, orc.layout.elemR, g, 1.0, False)
    # layout: zero exactly where the reference ELL has no column
    mask = orc.layout.colIds == oracle.INVALID
    assert np.all(S[mask] == 0) and np.all(R[mask] == 0)
    assert rel_err(S, So) < 2e-7
    assert rel_err(R, Ro) < 2e-7


@pytest.mark.parametrize("refine", [0.0, 1e-10])
def test_forward_2d_voltages(refine):
    import oracle
    import mpflow_gb300 as mp
    torch = _torch()
    mesh, src, orc = make_setup(rings=30, ports=16)
    g = inclusion_sigma(mesh, seed=0)
    Vo, Jo, _ = oracle.eit_forward(orc, g, tol=1e-13)
    model = mp.EIT(mesh, src, 1.0)
    V, J = model.solve(torch.tensor(g, dtype=torch.float32, device="cuda"),
                       mp.SolveOptions(tol=1e-7, refine_tol=refine), jacobian=True)
    V = V[0].cpu().numpy().astype(np.float64)
    J = J[0].cpu().numpy().astype(np.float64)
    tolV = 1e-5 if refine else 1e-4
    assert rel_err(V, Vo) < tolV, rel_err(V, Vo)
    assert rel_err(J, Jo) < 1e-4, rel_err(J, Jo)


def test_forward_2p5d_refined():
    import oracle
    import mpflow_gb300 as mp
    torch = _torch()
    mesh, src, orc = make_setup(rings=16, ports=32, width=0.1, components=8, height=4.0)
    rng = np.random.default_rng(1)
    g = np.exp(0.3 * rng.standard_normal(mesh.elements.shape[0]))
    Vo, Jo, Fo = oracle.eit_forward(orc, g, tol=1e-13)
    model = mp.EIT(mesh, src, 1.0, components=8, height=4.0)
    V, J = model.solve(torch.tensor(g, dtype=torch.float32, device="cuda"),
                       mp.SolveOptions(tol=1e-6, refine_tol=1e-10), jacobian=True)
    st = model.last_stats
    assert st.max_rel_residual <= 1e-10
    assert rel_err(V[0].cpu().numpy(), Vo) < 1e-5
    assert rel_err(J[0].cpu().numpy(), Jo) < 1e-4
    F = model.fields(1)[0].cpu().numpy()  # (C, Md+Mm, dataRows)
    n = mesh.nodes.shape[0]
    scale = np.abs(Fo[0]).max()
    for c in range(8):
        # harmonic 4 has beta = 2 sin(pi)/(4 pi) ~ 1e-17: its field is rounding noise
        err = np.abs(F[c][:, :n].T - Fo[c]).max() / scale
        assert err < 1e-6, (c, err)


def test_batched_frames_match_single():
    import mpflow_gb300 as mp
    torch = _torch()
    mesh, src, orc = make_setup(rings=16, ports=16, components=3, height=2.0)
    gs = np.stack([inclusion_sigma(mesh, seed=s) for s in range(4)])
    model = mp.EIT(mesh, src, 1.0, components=3, height=2.0)
    opts = mp.SolveOptions(tol=1e-7, refine_tol=1e-10)
    Vb = model.solve(torch.tensor(gs, dtype=torch.float32, device="cuda"), opts).cpu().numpy()
    for s in range(4):
        V1 = model.solve(torch.tensor(gs[s], dtype=torch.float32, device="cuda"), opts).cpu().numpy()[0]
        assert rel_err(Vb[s], V1) < 1e-6


def test_gram_split_bf16_accuracy():
    import mpflow_gb300 as mp
    torch = _torch()
    rng = np.random.default_rng(7)
    A = rng.standard_normal((2, 256, 640)).astype(np.float32)
    C = mp.gram_split_bf16(torch.tensor(A, device="cuda")).cpu().numpy()
    Ad = A.astype(np.float64)
    ref = np.einsum("bik,bjk->bij", Ad, Ad)
    # split hi+lo BF16 with FP32 accumulation: ~1e-5 normwise
    err = np.abs(C - ref).max() / np.abs(ref).max()
    assert err < 3e-5, err


@pytest.mark.parametrize("n,nrhs", [(32, 1), (256, 1), (1024, 1), (160, 3), (5120, 2)])
def test_cholesky_f64(n, nrhs):
    """Batched FP64 Cholesky factor + solve; n = 5120 takes the solve's
    shared-memory opt-in (x above 38 KB)."""
    import mpflow_gb300 as mp
    torch = _torch()
    rng = np.random.default_rng(5 + n)
    if n <= 1024:
        X = rng.standard_normal((3, n, n))
        A = np.einsum("bij,bkj->bik", X, X) / n
    else:  # symmetric, diagonally dominant
        B = rng.standard_normal((3, n, n)) / n
        A = B + B.transpose(0, 2, 1) + np.eye(n)[None] * (1.0 + rng.random((3, 1, n)))
    b = rng.standard_normal((3, nrhs, n))
    At = torch.tensor(A, device="cuda")
    Bt = torch.tensor(b, device="cuda")
    info = mp.cholesky_solve_f64(At, Bt, shift=0.5)
    assert int(info.abs().sum()) == 0
    x = Bt.cpu().numpy()
    for k in range(3):
        for c in range(nrhs):
            ref = np.linalg.solve(A[k] + 0.5 * np.eye(n), b[k, c])
            assert rel_err(x[k, c], ref) < 1e-10


def test_gn_step_matches_oracle_dual():
    import oracle
    import mpflow_gb300 as mp
    torch = _torch()
    mesh, src, orc = make_setup(rings=20, ports=16)
    g_true = inclusion_sigma(mesh, seed=0)
    Vmeas, _, _ = oracle.eit_forward(orc, g_true, tol=1e-13, want_jacobian=False)
    g0 = np.ones(mesh.elements.shape[0])
    V0, J0, _ = oracle.eit_forward(orc, g0, tol=1e-13)
    lam = 1e-2
    y = oracle.flatten_measurement(Vmeas, orc) - oracle.flatten_measurement(V0, orc)
    d_ref = oracle.inverse_dual(J0, y, 1.0, lam)
    model = mp.EIT(mesh, src, 1.0)
    gt = torch.ones((1, mesh.elements.shape[0]), dtype=torch.float32, device="cuda")
    vm = torch.tensor(Vmeas[None], dtype=torch.float32, device="cuda")  # (frames, Mm, Md) as solve() returns
    res = model.gn_step(gt, vm, lam, mp.SolveOptions(tol=1e-7, refine_tol=1e-10))
    d = gt[0].cpu().numpy() - 1.0
    assert abs(res[0] - np.linalg.norm(y) / np.linalg.norm(oracle.flatten_measurement(Vmeas, orc))) < 1e-5
    assert rel_err(d, d_ref) < 2e-3, rel_err(d, d_ref)


def test_config1_gn_step_at_spec():
    """Configuration 1 as specified: the 30-ring disk (2791 nodes, 5400
    triangles), 16 electrodes 0.1 rad wide, adjacent drive (1 mA) and
    measurement, 1 S/m with one 0.1 S/m inclusion of radius 0.2 centred in
    r < 0.6 (seed 0), 2D, CG tolerance 1e-6, one Gauss-Newton step from the
    homogeneous start with lambda = 1e-2, against the oracle's FP64 dual step
    (src/solver/solver.cpp:196-225, src/solver/inverse.cpp:60-238)."""
    import oracle
    import mpflow_gb300 as mp
    torch = _torch()
    mesh, src, orc = make_setup(rings=30, ports=16, width=0.1)
    assert mesh.nodes.shape[0] == 2791 and mesh.elements.shape[0] == 5400
    g_true = inclusion_sigma(mesh, seed=0)
    Vmeas, _, _ = oracle.eit_forward(orc, g_true, tol=1e-13, want_jacobian=False)
    g0 = np.ones(mesh.elements.shape[0])
    V0, J0, _ = oracle.eit_forward(orc, g0, tol=1e-13)
    lam = 1e-2
    y = oracle.flatten_measurement(Vmeas, orc) - oracle.flatten_measurement(V0, orc)
    d_ref = oracle.inverse_dual(J0, y, 1.0, lam)
    model = mp.EIT(mesh, src, 1.0)
    gt = torch.ones((1, mesh.elements.shape[0]), dtype=torch.float32, device="cuda")
    vm = torch.tensor(Vmeas[None], dtype=torch.float32, device="cuda")
    res = model.gn_step(gt, vm, lam, mp.SolveOptions(tol=1e-6))
    d = gt[0].cpu().numpy() - 1.0
    assert abs(res[0] - np.linalg.norm(y) / np.linalg.norm(oracle.flatten_measurement(Vmeas, orc))) < 1e-4
    assert rel_err(d, d_ref) < 2e-3, rel_err(d, d_ref)


def test_exact_jacobian_2p5d_matches_oracle():
    import oracle
    import mpflow_gb300 as mp
    torch = _torch()
    mesh, src, orc = make_setup(rings=16, ports=16, components=4, height=2.0)
    rng = np.random.default_rng(3)
    g = np.exp(0.3 * rng.standard_normal(mesh.elements.shape[0]))
    Vo, Jo, _ = oracle.eit_forward(orc, g, tol=1e-13, exact=True)
    model = mp.EIT(mesh, src, 1.0, components=4, height=2.0, exact_jacobian=True)
    V, J = model.solve(torch.tensor(g, dtype=torch.float32, device="cuda"),
                       mp.SolveOptions(tol=1e-5, refine_tol=1e-10), jacobian=True)
    assert rel_err(V[0].cpu().numpy(), Vo) < 1e-5
    assert rel_err(J[0].cpu().numpy(), Jo) < 1e-4


def test_identity_measurement_pattern_constant_mode():
    """Identity measurement patterns are not zero-sum, so the voltages see the
    constant mode of the Neumann harmonic (the reference's (A + 1 1^T) system)."""
    import oracle
    import mpflow_gb300 as mp
    torch = _torch()
    mesh = mp.IrregularMesh.ring(16)
    pr = mp.Ports.circularBoundary(16, 0.1, mesh)
    drive = mp.adjacent_pattern(16)
    meas = np.eye(16)
    src = mp.Sources(mp.OPEN, 1e-3, pr, drive, meas)
    orc = oracle.Setup(mesh.nodes, mesh.elements, mesh.edges, mesh.boundary, pr.edges, drive, meas,
                       np.full(16, 1e-3), components=2, height=2.0)
    g = inclusion_sigma(mesh, seed=5)
    Vo, Jo, _ = oracle.eit_forward(orc, g, tol=1e-13)
    model = mp.EIT(mesh, src, 1.0, components=2, height=2.0)
    V, J = model.solve(torch.tensor(g, dtype=torch.float32, device="cuda"),
                       mp.SolveOptions(tol=1e-5, refine_tol=1e-10), jacobian=True)
    assert model.info["unique_columns"] == 32
    assert rel_err(V[0].cpu().numpy(), Vo) < 1e-5
    assert rel_err(J[0].cpu().numpy(), Jo) < 1e-4


def test_warm_start_reproduces_cold_solve():
    import mpflow_gb300 as mp
    torch = _torch()
    mesh, src, orc = make_setup(rings=24, ports=16, components=3, height=2.0)
    gs = torch.tensor(np.stack([inclusion_sigma(mesh, seed=s) for s in range(3)]), dtype=torch.float32,
                      device="cuda")
    model = mp.EIT(mesh, src, 1.0, components=3, height=2.0)
    V1 = model.solve(gs, mp.SolveOptions(tol=1e-7)).cpu().numpy()
    cold = model.last_stats.iterations
    V2 = model.solve(gs * 1.01, mp.SolveOptions(tol=1e-7, warm_start=True)).cpu().numpy()
    warm = model.last_stats.iterations
    # linear parametrisation: V scales as 1/sigma
    assert rel_err(V2 * 1.01, V1) < 1e-5
    assert warm < cold


def test_iteration_cap_is_reported():
    import mpflow_gb300 as mp
    torch = _torch()
    mesh, src, orc = make_setup(rings=16)
    model = mp.EIT(mesh, src, 1.0)
    g = torch.ones((1, mesh.elements.shape[0]), device="cuda")
    with pytest.raises(mp.MpfError) as ei:
        model.solve(g, mp.SolveOptions(tol=1e-7, max_iter=2, check_every=1))
    assert ei.value.status == 4
    model.solve(g, mp.SolveOptions(tol=1e-7, max_iter=2, check_every=1), raise_on_noconv=False)
    assert model.last_stats.not_converged > 0


def test_gn_solve_reaches_target():
    import oracle
    import mpflow_gb300 as mp
    torch = _torch()
    mesh, src, orc = make_setup(rings=24, ports=16, logarithmic=True)
    E = mesh.elements.shape[0]
    model = mp.EIT(mesh, src, 1.0, logarithmic=True)
    vt = np.stack([10 * np.log10(inclusion_sigma(mesh, seed=s, value=v)) for s, v in ((0, 0.2), (1, 5.0))])
    Vm = model.solve(torch.tensor(vt, dtype=torch.float32, device="cuda"), mp.SolveOptions(tol=1e-6, refine_tol=1e-10))
    _, J0 = model.solve(torch.zeros((1, E), device="cuda"), mp.SolveOptions(tol=1e-6), jacobian=True)
    lam = 2e-2 * float(J0.norm() / np.sqrt(J0.shape[1]))
    g = torch.zeros((2, E), device="cuda")
    iters, res, st = model.gn_solve(g, Vm, lam, target=5e-4, max_iters=10, options=mp.SolveOptions(tol=1e-6))
    assert st.frames_converged == 2 and (res <= 5e-4).all()
    assert (iters >= 1).all()
    # the first GN update agrees with the oracle's dual step from the same start
    g1 = torch.zeros((1, E), device="cuda")
    model.gn_step(g1, Vm[0:1], lam, mp.SolveOptions(tol=1e-7, refine_tol=1e-10))
    V0, Jo, _ = oracle.eit_forward(orc, np.zeros(E), tol=1e-13)
    y = Vm[0].cpu().numpy().astype(np.float64).T.reshape(-1) - oracle.flatten_measurement(V0, orc)
    d_ref = oracle.inverse_dual(Jo, y, 1.0, lam)
    assert rel_err(g1[0].cpu().numpy(), d_ref) < 5e-3


def test_profile_cg_reports_bandwidth():
    import mpflow_gb300 as mp
    torch = _torch()
    mesh, src, orc = make_setup(rings=24)
    model = mp.EIT(mesh, src, 1.0)
    n0 = mp.lib().mpf_kernel_launches()
    ms, by = model.profile_cg(torch.ones((2, mesh.elements.shape[0]), device="cuda"), reps=3)
    assert (ms > 0).all() and (by > 0).all()
    assert mp.lib().mpf_kernel_launches() - n0 >= 10


@pytest.mark.parametrize("ports,components", [(16, 2), (32, 3)])
def test_every_cg_variant_matches_oracle(ports, components):
    """Every launch shape the autotuner may pick gives the oracle's voltages
    (2.5D model: one Neumann harmonic plus regular ones)."""
    import oracle
    import mpflow_gb300 as mp
    torch = _torch()
    mesh, src, orc = make_setup(rings=20, ports=ports, components=components, height=2.0)
    g = inclusion_sigma(mesh, seed=5)
    Vo, _, _ = oracle.eit_forward(orc, g, tol=1e-13)
    model = mp.EIT(mesh, src, 1.0, components=components, height=2.0)
    gt = torch.tensor(g, dtype=torch.float32, device="cuda")
    model.solve(gt, mp.SolveOptions(tol=1e-7))
    tuned = model.cg_variants(1)
    assert (tuned >= 0).all() and tuned[0] < 144 and (tuned[1:] < 36).all()
    tried = 0
    # 9 lane/row-step variants x 1, 2, 4, 8 tiles per block; SpMM codes 36..71
    # are the form with per-warp cp.async staging of the slots, 72..107 and
    # 108..143 the tile-staged form (own and halo rows copied in bulk) with 2
    # and 3 stages
    for v in range(144):
        shapes = [v, v, v] if v < 36 else [v, int(tuned[1]), int(tuned[2])]
        try:
            model.cg_variants(1, set=shapes)
        except mp.MpfError as e:
            assert e.status == 1
            continue
        tried += 1
        V = model.solve(gt, mp.SolveOptions(tol=1e-7))[0].cpu().numpy().astype(np.float64)
        assert rel_err(V, Vo) < 1e-4, (v, rel_err(V, Vo))
    assert tried >= 70
    model.cg_variants(1, set=[-1, -1, -1])
    assert (model.cg_variants(1) == tuned).all()


@pytest.mark.parametrize("refine", [0.0, 1e-10])
def test_two_level_preconditioner_matches_oracle(refine):
    """The two-level preconditioner gives the oracle's voltages and Jacobian
    (2.5D, Neumann and regular harmonics) in fewer iterations than Jacobi."""
    import oracle
    import mpflow_gb300 as mp
    torch = _torch()
    mesh, src, orc = make_setup(rings=30, ports=16, components=3, height=2.0)
    g = inclusion_sigma(mesh, seed=4)
    Vo, Jo, _ = oracle.eit_forward(orc, g, tol=1e-13)
    model = mp.EIT(mesh, src, 1.0, components=3, height=2.0)
    gt = torch.tensor(g, dtype=torch.float32, device="cuda")
    iters = {}
    for pc in ("jacobi", "two-level"):
        V, J = model.solve(gt, mp.SolveOptions(tol=1e-7, refine_tol=refine, preconditioner=pc), jacobian=True)
        iters[pc] = model.last_stats.iterations
        tolV = 1e-5 if refine else 1e-4
        assert rel_err(V[0].cpu().numpy(), Vo) < tolV, (pc, rel_err(V[0].cpu().numpy(), Vo))
        assert rel_err(J[0].cpu().numpy(), Jo) < 1e-4, (pc, rel_err(J[0].cpu().numpy(), Jo))
    assert iters["two-level"] < 0.6 * iters["jacobi"], iters


def test_two_level_warm_start_and_gn():
    import mpflow_gb300 as mp
    torch = _torch()
    mesh, src, orc = make_setup(rings=24, ports=16, components=3, height=2.0, logarithmic=True)
    E = mesh.elements.shape[0]
    model = mp.EIT(mesh, src, 1.0, components=3, height=2.0, logarithmic=True)
    vt = np.stack([10 * np.log10(inclusion_sigma(mesh, seed=s, value=v)) for s, v in ((0, 0.2), (1, 5.0))])
    Vm = model.solve(torch.tensor(vt, dtype=torch.float32, device="cuda"),
                     mp.SolveOptions(tol=1e-6, refine_tol=1e-10))
    _, J0 = model.solve(torch.zeros((1, E), device="cuda"), mp.SolveOptions(tol=1e-6), jacobian=True)
    lam = 2e-2 * float(J0.norm() / np.sqrt(J0.shape[1]))
    res = {}
    for pc in ("jacobi", "two-level"):
        g = torch.zeros((2, E), device="cuda")
        iters, r, st = model.gn_solve(g, Vm, lam, target=5e-4, max_iters=10,
                                      options=mp.SolveOptions(tol=1e-6, preconditioner=pc))
        assert st.frames_converged == 2, pc
        res[pc] = (g.cpu().numpy(), st.cg_iterations)
    # same reconstruction, fewer CG iterations
    assert rel_err(res["two-level"][0], res["jacobi"][0]) < 1e-2
    assert res["two-level"][1] < res["jacobi"][1]


def test_homogeneous_field_warm_start():
    """warm_start='homogeneous' reproduces the cold solve with fewer iterations."""
    import mpflow_gb300 as mp
    torch = _torch()
    mesh, src, orc = make_setup(rings=24, ports=16, components=3, height=2.0, logarithmic=True)
    model = mp.EIT(mesh, src, 1.0, components=3, height=2.0, logarithmic=True)
    g = torch.tensor(np.stack([10 * np.log10(inclusion_sigma(mesh, seed=s)) for s in range(3)]),
                     dtype=torch.float32, device="cuda")
    for pc in ("jacobi", "two-level"):
        V1 = model.solve(g, mp.SolveOptions(tol=1e-7, preconditioner=pc)).cpu().numpy()
        cold = model.last_stats.iterations
        V2 = model.solve(g, mp.SolveOptions(tol=1e-7, preconditioner=pc, warm_start="homogeneous")).cpu().numpy()
        assert rel_err(V2, V1) < 1e-5
        assert model.last_stats.iterations < cold
        # the homogeneous distribution itself needs no iterations from its own fields
        model.solve(torch.zeros_like(g), mp.SolveOptions(tol=1e-6, preconditioner=pc, warm_start="homogeneous"))
        assert model.last_stats.iterations <= 1


@pytest.mark.parametrize("kind", ["identity", "noser", "laplacian"])
def test_inverse_regularisers_match_oracle(kind):
    """mpf_inverse_solve (solver::Inverse) for two parallel images against the
    FP64 oracle solve of the same regularised system."""
    import oracle
    import mpflow_gb300 as mp
    torch = _torch()
    mesh, src, orc = make_setup(rings=16, ports=16)
    E = mesh.elements.shape[0]
    model = mp.EIT(mesh, src, 1.0)
    opts = mp.SolveOptions(tol=1e-7, refine_tol=1e-10)
    ref = torch.ones((1, E), device="cuda")
    calc1, J = model.solve(ref, opts, jacobian=True)
    gs = torch.tensor(np.stack([inclusion_sigma(mesh, seed=s) for s in (1, 2)]), dtype=torch.float32, device="cuda")
    meas = model.solve(gs, opts)
    calc = calc1.expand(2, -1, -1).contiguous()
    Jn = J[0].cpu().numpy().astype(np.float64)
    # factors that regularise each R to a comparable strength: (ref factor)^2 R
    # adds about a tenth of J^T J's mean diagonal
    djj = float((Jn ** 2).sum(axis=0).mean())
    if kind == "identity":
        factor = np.sqrt(0.1 * djj)
    elif kind == "noser":
        factor = np.sqrt(0.1)
    else:
        factor = np.sqrt(0.1 * djj / float(np.diag(oracle.laplacian_gram(mesh.nodes, mesh.elements)).mean()))
    out = model.inverse(J[0], calc, meas, factor, kind).cpu().numpy()
    # oracle on the same J and data (J rows in the library's d * MP + m order)
    Y = np.stack([oracle.flatten_measurement(meas[i].cpu().numpy().astype(np.float64), orc)
                  - oracle.flatten_measurement(calc[i].cpu().numpy().astype(np.float64), orc) for i in range(2)], 1)
    X = oracle.inverse_regularised(Jn, Y, 1.0, factor, kind, mesh.nodes, mesh.elements)
    for i in range(2):
        assert rel_err(out[i], X[:, i]) < 2e-3, (kind, i, rel_err(out[i], X[:, i]))


@pytest.mark.parametrize("components,height,pc", [(1, 1.0, "jacobi"), (3, 2.0, "jacobi"), (3, 2.0, "two-level")])
def test_fixed_sources_match_oracle(components, height, pc):
    """Voltage sources (Dirichlet rows on the port nodes, currents measured)
    against the oracle's dense solve of the reference's system."""
    import oracle
    import mpflow_gb300 as mp
    torch = _torch()
    mesh, src, orc = make_setup(rings=16, ports=16, components=components, height=height, current=1.0)
    fixed = mp.Sources(mp.FIXED, 1.0, src.ports, src.drivePattern, src.measurementPattern)
    g = inclusion_sigma(mesh, seed=6)
    Vo, Jo, Fo = oracle.eit_forward_fixed(orc, g)
    model = mp.EIT(mesh, fixed, 1.0, components=components, height=height)
    V, J = model.solve(torch.tensor(g, dtype=torch.float32, device="cuda"),
                       mp.SolveOptions(tol=1e-8, preconditioner=pc), jacobian=True)
    assert rel_err(V[0].cpu().numpy(), Vo) < 1e-4, rel_err(V[0].cpu().numpy(), Vo)
    assert rel_err(J[0].cpu().numpy(), Jo) < 1e-4, rel_err(J[0].cpu().numpy(), Jo)
    n = mesh.nodes.shape[0]
    Fg = model.fields(1)[0].cpu().numpy()
    for c in range(components):
        err = np.abs(Fg[c][:, :n].T - Fo[c]).max() / np.abs(Fo[c]).max()
        assert err < 1e-5, (c, err)


def test_profile_gram_hook():
    """mpf_profile_gram (the bench's J J^T timing) runs and rejects bad shapes."""
    import mpflow_gb300 as mp
    ms = mp.profile_gram(2, 256, 512, reps=2)
    assert 0.0 < ms < 1e3
    with pytest.raises(mp.MpfError):
        mp.profile_gram(1, 100, 512)


def test_profile_fem_hook():
    """mpf_eit_profile_fem (the bench's assembly / Jacobian timing)."""
    import mpflow_gb300 as mp
    torch = _torch()
    mesh, src, _ = make_setup(rings=16, ports=16, components=2, height=2.0)
    model = mp.EIT(mesh, src, 1.0, components=2, height=2.0)
    g = torch.ones((2, mesh.elements.shape[0]), device="cuda")
    ms, by = model.profile_fem(g, reps=2)
    assert (ms > 0).all() and (by > 0).all()
    assert by[1] > by[0]  # the Jacobian writes rowsJ x E per frame
