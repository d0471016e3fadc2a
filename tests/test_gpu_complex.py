"""Complex admittivity (mpf_eit_forward_complex) against the FP64 oracle's
complex forward model and against the real path, through the C ABI."""
import numpy as np
import pytest

from conftest import inclusion_sigma, make_setup

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _complex_frames(mesh, count, seed, logarithmic):
    """Conductivity with an inclusion plus a permittivity-like imaginary part."""
    rng = np.random.default_rng(seed)
    out = []
    for f in range(count):
        sig = inclusion_sigma(mesh, seed=seed + f)
        eps = 0.1 + 0.2 * rng.random(mesh.elements.shape[0])
        g = sig + 1j * eps * sig
        out.append(10.0 * np.log10(g) if logarithmic else g)
    return np.stack(out)


@pytest.mark.parametrize("logarithmic", [False, True])
def test_complex_forward_matches_oracle(logarithmic):
    import oracle
    import torch
    import mpflow_gb300 as mp
    mesh, src, orc = make_setup(rings=16, ports=16, components=3, height=2.0, logarithmic=logarithmic)
    g = _complex_frames(mesh, 2, seed=3, logarithmic=logarithmic)
    model = mp.EIT(mesh, src, 1.0, components=3, height=2.0, logarithmic=logarithmic)
    V, J = model.solve_complex(torch.tensor(g, dtype=torch.complex64, device="cuda"),
                               mp.SolveOptions(tol=1e-7, solver="bicgstab"), jacobian=True)
    assert model.last_stats.not_converged == 0 and model.last_stats.iterations > 0
    for f in range(2):
        Vo, Jo = oracle.eit_forward_complex(orc, g[f], want_jacobian=True)
        assert np.abs(Vo.imag).max() > 1e-3 * np.abs(Vo.real).max()  # a genuinely complex case
        assert rel_err(V[f].cpu().numpy(), Vo) < 1e-4, f
        assert J[f].shape == Jo.shape
        assert rel_err(J[f].cpu().numpy(), Jo) < 1e-4, f


def test_complex_fields_match_oracle():
    """mpf_eit_fields_complex (EIT::fields of the complex instantiations):
    every component's complex potentials, in the reference's convention for
    the Neumann harmonic, against the oracle's FP64 fields."""
    import oracle
    import torch
    import mpflow_gb300 as mp
    mesh, src, orc = make_setup(rings=16, ports=16, components=3, height=2.0)
    g = _complex_frames(mesh, 2, seed=5, logarithmic=False)
    model = mp.EIT(mesh, src, 1.0, components=3, height=2.0)
    with pytest.raises(mp.MpfError):
        model.fields_complex(1)  # no complex solve yet
    model.solve_complex(torch.tensor(g, dtype=torch.complex64, device="cuda"),
                        mp.SolveOptions(tol=1e-7, solver="bicgstab"))
    Fz = model.fields_complex(2).cpu().numpy()  # (frames, C, Md+Mm, data_rows)
    n = mesh.nodes.shape[0]
    for f in range(2):
        _, Fo = oracle.eit_forward_complex(orc, g[f], want_fields=True)
        scale = np.abs(Fo[0]).max()
        for c in range(3):
            err = np.abs(Fz[f, c][:, :n].T - Fo[c]).max() / scale
            assert err < 1e-5, (f, c, err)


def test_complex_with_real_values_equals_real_solve():
    import torch
    import mpflow_gb300 as mp
    mesh, src, _ = make_setup(rings=20, ports=32, width=0.1, components=4, height=4.0)
    g = np.stack([inclusion_sigma(mesh, seed=s) for s in range(3)])
    model = mp.EIT(mesh, src, 1.0, components=4, height=4.0)
    Vr, Jr = model.solve(torch.tensor(g, dtype=torch.float32, device="cuda"), mp.SolveOptions(tol=1e-7),
                         jacobian=True)
    Vz, Jz = model.solve_complex(torch.tensor(g, dtype=torch.complex64, device="cuda"),
                                 mp.SolveOptions(tol=1e-7, solver="bicgstab"), jacobian=True)
    Vr, Jr = Vr.cpu().numpy(), Jr.cpu().numpy()
    Vz, Jz = Vz.cpu().numpy(), Jz.cpu().numpy()
    assert rel_err(Vz.real, Vr) < 2e-5
    assert np.abs(Vz.imag).max() <= 1e-6 * np.abs(Vr).max()
    assert rel_err(Jz.real, Jr) < 5e-5
    assert np.abs(Jz.imag).max() <= 1e-6 * np.abs(Jr).max()


def test_complex_rejects_unsupported_options():
    import torch
    import mpflow_gb300 as mp
    mesh, src, _ = make_setup(rings=12, ports=16, width=0.2)
    model = mp.EIT(mesh, src, 1.0)
    g = torch.ones((1, mesh.elements.shape[0]), dtype=torch.complex64, device="cuda")
    for opts in (mp.SolveOptions(refine_tol=1e-9), mp.SolveOptions(warm_start=True)):
        with pytest.raises(mp.MpfError) as e:
            model.solve_complex(g, opts)
        assert e.value.status == 8


@pytest.mark.parametrize("kind", ["identity", "noser", "laplacian"])
def test_complex_inverse_matches_oracle(kind):
    """mpf_inverse_solve_complex (solver::Inverse on thrust::complex<float>)
    for two images against the FP64 complex solve of the same regularised
    system with the plain transpose (numpy J.T, as the reference's
    CUBLAS_OP_T)."""
    import oracle
    import torch
    import mpflow_gb300 as mp
    mesh, src, orc = make_setup(rings=16, ports=16, components=3, height=2.0)
    E = mesh.elements.shape[0]
    model = mp.EIT(mesh, src, 1.0, components=3, height=2.0)
    opts = mp.SolveOptions(tol=1e-7, solver="bicgstab")
    ref = torch.full((1, E), 1.0 + 0.15j, dtype=torch.complex64, device="cuda")
    calc1, J = model.solve_complex(ref, opts, jacobian=True)
    g = _complex_frames(mesh, 2, seed=7, logarithmic=False)
    meas = model.solve_complex(torch.tensor(g, dtype=torch.complex64, device="cuda"), opts)
    calc = calc1.expand(2, -1, -1).contiguous()
    Jn = J[0].cpu().numpy().astype(np.complex128)
    assert np.abs(Jn.imag).max() > 1e-3 * np.abs(Jn.real).max()
    djj = float((np.abs(Jn) ** 2).sum(axis=0).mean())
    if kind == "identity":
        factor = np.sqrt(0.1 * djj)
    elif kind == "noser":
        factor = np.sqrt(0.1)
    else:
        factor = np.sqrt(0.1 * djj / float(np.diag(oracle.laplacian_gram(mesh.nodes, mesh.elements)).mean()))
    out = model.inverse_complex(J[0], calc, meas, factor, kind).cpu().numpy()

    def flat(V):
        V = V.cpu().numpy().astype(np.complex128)
        return oracle.flatten_measurement(V.real, orc) + 1j * oracle.flatten_measurement(V.imag, orc)

    Y = np.stack([flat(meas[i]) - flat(calc[i]) for i in range(2)], 1)
    X = oracle.inverse_regularised(Jn, Y, 1.0, factor, kind, mesh.nodes, mesh.elements)
    assert np.abs(X.imag).max() > 1e-3 * np.abs(X.real).max()
    for i in range(2):
        assert rel_err(out[i], X[:, i]) < 1e-5, (kind, i, rel_err(out[i], X[:, i]))
