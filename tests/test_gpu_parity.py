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
    mesh, src, orc = make_setup(rings=14)
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
    for c in range(8):
        assert rel_err(F[c][:, :n].T, Fo[c]) < 1e-5, c


def test_batched_frames_match_single():
    import mpflow_gb300 as mp
    torch = _torch()
    mesh, src, orc = make_setup(rings=12, ports=16, components=3, height=2.0)
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


def test_cholesky_f64():
    import mpflow_gb300 as mp
    torch = _torch()
    rng = np.random.default_rng(5)
    n = 256
    X = rng.standard_normal((3, n, n))
    A = np.einsum("bij,bkj->bik", X, X) / n
    b = rng.standard_normal((3, 1, n))
    At = torch.tensor(A, device="cuda")
    Bt = torch.tensor(b, device="cuda")
    info = mp.cholesky_solve_f64(At, Bt, shift=0.5)
    assert int(info.abs().sum()) == 0
    x = Bt.cpu().numpy()
    for k in range(3):
        ref = np.linalg.solve(A[k] + 0.5 * np.eye(n), b[k, 0])
        assert rel_err(x[k, 0], ref) < 1e-10


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
    vm = torch.tensor(Vmeas.T.reshape(1, -1), dtype=torch.float32, device="cuda")  # column-major Mm x Md
    res = model.gn_step(gt, vm, lam, mp.SolveOptions(tol=1e-7, refine_tol=1e-10))
    d = gt[0].cpu().numpy() - 1.0
    assert abs(res[0] - np.linalg.norm(y) / np.linalg.norm(oracle.flatten_measurement(Vmeas, orc))) < 1e-5
    assert rel_err(d, d_ref) < 2e-3, rel_err(d, d_ref)
