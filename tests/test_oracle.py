"""Known-answer checks of the FP64 oracle (CPU only).

The reference ships no tests or golden vectors, so the oracle is pinned by
properties that the reference's mathematics must satisfy and by the committed
fixtures in tests/golden (generated from this oracle by make_golden.py).
"""
import os

import numpy as np
import pytest

from conftest import inclusion_sigma, make_setup

import oracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_padding_rule():
    # src/numeric/matrix.cpp:49-55 with roundTo (mathematics.h:42-44)
    assert [oracle.data_rows(n) for n in (1, 2, 15, 16, 17, 32, 2791, 19441)] == \
        [1, 16, 16, 16, 32, 32, 2800, 19456]


def test_p1_integrals_analytic():
    mesh, _, orc = make_setup(rings=6, ports=4, width=0.5)
    K, M = orc.K, orc.M
    # rows of the stiffness matrix sum to zero (constants are in the kernel)
    assert np.abs(K.sum(axis=2)).max() < 1e-13
    # mass integrates to the triangle area; total = area of the 36-gon
    assert abs(M.sum() - 0.5 * 36 * np.sin(2 * np.pi / 36)) < 1e-13
    # stiffness is symmetric positive semidefinite per element
    assert np.abs(K - K.transpose(0, 2, 1)).max() < 1e-14
    assert np.linalg.eigvalsh(K).min() > -1e-13


def test_ell_layout_insertion_order():
    mesh, _, orc = make_setup(rings=5, ports=4, width=0.5)
    lay = orc.layout
    # every used slot of a row holds a distinct neighbour; the diagonal is present
    for row in range(mesh.nodes.shape[0]):
        ids = lay.colIds[row][lay.colIds[row] != oracle.INVALID]
        assert len(set(ids.tolist())) == len(ids)
        assert row in ids
    # the first element's nodes were inserted first (src/fem/equation.cpp:133-138)
    e0 = mesh.elements[0]
    for i in range(3):
        assert list(lay.colIds[e0[i]][:3]) == list(e0)


def test_forward_reciprocity_and_conservation():
    mesh, _, orc = make_setup(rings=16)
    g = inclusion_sigma(mesh, seed=2)
    V, J, _ = oracle.eit_forward(orc, g, tol=1e-13)
    # adjacent drive == adjacent measurement: V is symmetric up to the current value
    Vs = V / 1e-3
    assert np.abs(Vs - Vs.T).max() / np.abs(Vs).max() < 1e-10
    # measurements around the ring sum to zero for every drive
    assert np.abs(V.sum(axis=0)).max() / np.abs(V).max() < 1e-12


def test_jacobian_homogeneity_and_fd():
    mesh, _, orc = make_setup(rings=16)
    rng = np.random.default_rng(0)
    g = 1.0 + 0.5 * rng.random(mesh.elements.shape[0])
    V, J, _ = oracle.eit_forward(orc, g, tol=1e-13)
    Vf = oracle.flatten_measurement(V, orc)
    # linear parametrisation, one harmonic: V is homogeneous of degree -1 in sigma
    assert np.abs(J @ g + Vf).max() / np.abs(Vf).max() < 1e-10
    d = rng.standard_normal(g.size) * 1e-4
    Vp, _, _ = oracle.eit_forward(orc, g + d, tol=1e-13, want_jacobian=False)
    Vm, _, _ = oracle.eit_forward(orc, g - d, tol=1e-13, want_jacobian=False)
    fd = (oracle.flatten_measurement(Vp, orc) - oracle.flatten_measurement(Vm, orc)) / 2
    assert np.abs(fd - J @ d).max() / np.abs(fd).max() < 1e-6


def test_exact_jacobian_matches_fd_in_2p5d():
    mesh, _, orc = make_setup(rings=8, width=0.2, components=4, height=2.0)
    rng = np.random.default_rng(1)
    g = 1.0 + 0.3 * rng.random(mesh.elements.shape[0])
    _, J, _ = oracle.eit_forward(orc, g, tol=1e-13, exact=True)
    d = rng.standard_normal(g.size) * 1e-4
    Vp, _, _ = oracle.eit_forward(orc, g + d, tol=1e-13, want_jacobian=False)
    Vm, _, _ = oracle.eit_forward(orc, g - d, tol=1e-13, want_jacobian=False)
    fd = (oracle.flatten_measurement(Vp, orc) - oracle.flatten_measurement(Vm, orc)) / 2
    assert np.abs(fd - J @ d).max() / np.abs(fd).max() < 1e-6
    # the reference's 2.5D Jacobian keeps only the stiffness term and is not the FD derivative
    _, Jr, _ = oracle.eit_forward(orc, g, tol=1e-13, exact=False)
    assert np.abs(fd - Jr @ d).max() / np.abs(fd).max() > 1e-2


def test_inverse_primal_equals_dual():
    mesh, _, orc = make_setup(rings=16)
    g = inclusion_sigma(mesh, seed=4)
    V, J, _ = oracle.eit_forward(orc, np.ones(mesh.elements.shape[0]), tol=1e-13)
    Vt, _, _ = oracle.eit_forward(orc, g, tol=1e-13, want_jacobian=False)
    y = oracle.flatten_measurement(Vt, orc) - oracle.flatten_measurement(V, orc)
    dp = oracle.inverse_primal(J, y, 1.0, 1e-2)
    dd = oracle.inverse_dual(J, y, 1.0, 1e-2)
    assert np.abs(dp - dd).max() / np.abs(dd).max() < 1e-9


def test_cholesky_reports_breakdown():
    A = np.array([[1.0, 2.0], [2.0, 1.0]], order="F")
    assert oracle.lib().orc_cholesky(2, oracle._p(A)) == 2


@pytest.mark.parametrize("name", ["config1_small", "config2_r40"])
def test_golden_fixture(name):
    """The oracle reproduces the committed fixture (regression pin)."""
    path = os.path.join(GOLDEN, f"{name}.npz")
    if not os.path.exists(path):
        pytest.skip("fixture not generated")
    z = np.load(path)
    extra = {"components": int(z["components"]), "height": float(z["height"])} if "components" in z.files else {}
    mesh, _, orc = make_setup(rings=int(z["rings"]), ports=int(z["ports"]), **extra)
    V, J, _ = oracle.eit_forward(orc, z["sigma"], tol=1e-13)
    assert np.abs(V - z["V"]).max() / np.abs(z["V"]).max() < 1e-10
    Jp = J @ z["probes"]
    assert np.abs(Jp - z["J_probe"]).max() / np.abs(z["J_probe"]).max() < 1e-9
    assert np.array_equal(orc.layout.colIds, z["colIds"])
    assert np.array_equal(orc.portEdges, z["portEdges"])


def test_fixed_source_oracle_jacobian_is_derivative():
    """Voltage sources, one harmonic: the reference's Jacobian formula equals the
    finite-difference derivative of the measured currents, and the current
    matrix is symmetric (reciprocity)."""
    import oracle
    from conftest import make_setup
    mesh, src, orc = make_setup(rings=16, ports=16, current=1.0)
    g = np.ones(mesh.elements.shape[0])
    V, J, _ = oracle.eit_forward_fixed(orc, g)
    assert np.abs(V - V.T).max() <= 1e-12 * np.abs(V).max()
    e, h = 57, 1e-4
    gp, gm = g.copy(), g.copy()
    gp[e] += h
    gm[e] -= h
    Vp, _, _ = oracle.eit_forward_fixed(orc, gp, want_jacobian=False)
    Vm, _, _ = oracle.eit_forward_fixed(orc, gm, want_jacobian=False)
    fd = oracle.flatten_measurement((Vp - Vm) / (2 * h), orc)
    assert np.abs(fd - J[:, e]).max() <= 1e-5 * np.abs(J[:, e]).max()


def test_bicgstab_oracle_matches_cg_oracle():
    """The two Krylov solvers of models::EIT give the same voltages and
    Jacobian; fields agree up to a constant on the Neumann harmonic (the
    reference's BiCGSTAB ignores dcFree)."""
    mesh, src, orc = make_setup(rings=16, ports=16, components=3, height=2.0)
    g = inclusion_sigma(mesh, seed=1)
    V1, J1, F1 = oracle.eit_forward(orc, g, tol=1e-13)
    V2, J2, F2 = oracle.eit_forward(orc, g, tol=1e-13, solver="bicgstab")
    assert np.abs(V1 - V2).max() <= 1e-11 * np.abs(V1).max()
    assert np.abs(J1 - J2).max() <= 1e-11 * np.abs(J1).max()
    for c in range(3):
        d = F1[c] - F2[c]
        assert np.abs(d - d.mean(axis=0)).max() <= 1e-11 * np.abs(F1[c]).max()
        if c > 0:
            assert np.abs(d).max() <= 1e-11 * np.abs(F1[c]).max()


def test_complex_oracle_reduces_to_real():
    """With zero imaginary part the complex forward model is the real one."""
    mesh, src, orc = make_setup(rings=12, ports=8, width=0.3, components=3, height=2.0)
    g = inclusion_sigma(mesh, seed=2)
    V, _, _ = oracle.eit_forward(orc, g, tol=1e-14, want_jacobian=False)
    Vz = oracle.eit_forward_complex(orc, g.astype(np.complex128))
    assert np.abs(Vz.imag).max() <= 1e-12 * np.abs(V).max()
    assert np.abs(Vz.real - V).max() <= 1e-9 * np.abs(V).max()


def test_complex_oracle_jacobian_reduces_to_real():
    mesh, src, orc = make_setup(rings=12, ports=8, width=0.3, components=2, height=2.0)
    g = inclusion_sigma(mesh, seed=4)
    _, J, _ = oracle.eit_forward(orc, g, tol=1e-14)
    _, Jz = oracle.eit_forward_complex(orc, g.astype(np.complex128), want_jacobian=True)
    assert np.abs(Jz.imag).max() <= 1e-12 * np.abs(J).max()
    assert np.abs(Jz.real - J).max() <= 1e-8 * np.abs(J).max()


def test_complex_inverse_dual_equals_primal():
    """The complex inverse's dual form: with the reference's plain
    transpose (CUBLAS_OP_T on complex data), J^T (J J^T + mu I)^-1 y equals
    (J^T J + mu I)^-1 J^T y for the complex symmetric systems, on the
    oracle's complex Jacobian."""
    mesh, _, orc = make_setup(rings=12, ports=8, width=0.3, components=2, height=2.0)
    E = mesh.elements.shape[0]
    g0 = np.full(E, 1.0 + 0.2j)
    V0, J = oracle.eit_forward_complex(orc, g0, want_jacobian=True)
    g = g0.copy()
    g[: E // 5] = 0.5 + 0.4j
    Vt = oracle.eit_forward_complex(orc, g, want_jacobian=False)

    def flat(V):
        return oracle.flatten_measurement(V.real, orc) + 1j * oracle.flatten_measurement(V.imag, orc)

    y = flat(Vt) - flat(V0)
    mu = 0.1 * float((np.abs(J) ** 2).sum(axis=0).mean())
    primal = oracle.inverse_regularised(J, y[:, None], 1.0, np.sqrt(mu), "identity")[:, 0]
    dual = J.T @ np.linalg.solve(J @ J.T + mu * np.eye(J.shape[0]), y)
    assert np.abs(primal.imag).max() > 1e-3 * np.abs(primal).max()
    assert np.abs(primal - dual).max() <= 1e-9 * np.abs(primal).max()


def test_mesh_refinement_convergence_homogeneous_disk():
    """Electrode voltages of the homogeneous disk converge under mesh
    refinement.  Six electrodes of width pi/6 start and end on boundary nodes
    at every even ring count, so only the discretisation changes between
    meshes; the differences of successive refinements must shrink at least
    like h (P1 elements: about h^2)."""
    Vs = []
    for rings in (6, 12, 24, 48):
        mesh, _, orc = make_setup(rings=rings, ports=6, width=np.pi / 6)
        V, _, _ = oracle.eit_forward(orc, np.ones(mesh.elements.shape[0]), tol=1e-13, want_jacobian=False)
        Vs.append(np.asarray(V, np.float64))
    d = [np.abs(Vs[k + 1] - Vs[k]).max() for k in range(3)]
    assert all(d[k + 1] < 0.5 * d[k] for k in range(2)), d
    assert np.abs(Vs[-1] - Vs[-2]).max() < 1e-2 * np.abs(Vs[-1]).max(), d


def test_complex_symmetric_cholesky_restatement():
    """The complex inverse factors J J^T + mu I as L L^T with complex L and
    no conjugation (zinverse.cu).  Restated here in FP64 numpy with the
    same column order, Smith's division and the principal square root from
    |z|, on a complex Gram of the oracle's complex Jacobian: L L^T
    reproduces the matrix and the solve matches numpy's."""
    mesh, _, orc = make_setup(rings=12, ports=8, width=0.3, components=2, height=2.0)
    E = mesh.elements.shape[0]
    _, J = oracle.eit_forward_complex(orc, np.full(E, 1.0 + 0.3j), want_jacobian=True)
    n = J.shape[0]
    mu = 0.05 * float((np.abs(J) ** 2).sum(axis=1).mean())
    A = J @ J.T + mu * np.eye(n)

    def zsqrt(z):
        r = abs(z)
        if z.real >= 0:
            t = np.sqrt(0.5 * (r + z.real))
            return complex(t, z.imag / (2 * t))
        t = np.sqrt(0.5 * (r - z.real))
        return complex(abs(z.imag) / (2 * t), np.copysign(t, z.imag))

    def zdiv(a, b):
        if abs(b.real) >= abs(b.imag):
            r = b.imag / b.real
            d = b.real + b.imag * r
            return complex((a.real + a.imag * r) / d, (a.imag - a.real * r) / d)
        r = b.real / b.imag
        d = b.imag + b.real * r
        return complex((a.real * r + a.imag) / d, (a.imag * r - a.real) / d)

    L = A.copy()
    for j in range(n):
        L[j, j] = zsqrt(L[j, j])
        for i in range(j + 1, n):
            L[i, j] = zdiv(L[i, j], L[j, j])
        L[j + 1:, j + 1:] -= np.tril(np.outer(L[j + 1:, j], L[j + 1:, j]))
    L = np.tril(L)
    assert np.abs(L @ L.T - A).max() <= 1e-12 * np.abs(A).max()
    b = np.random.default_rng(2).standard_normal(n) + 1j * np.random.default_rng(3).standard_normal(n)
    z = np.linalg.solve(L, b)            # forward: L z = b
    x = np.linalg.solve(L.T, z)          # backward: L^T x = z (plain transpose)
    assert np.abs(x - np.linalg.solve(A, b)).max() <= 1e-9 * np.abs(x).max()


def test_golden_fixture_complex():
    """The complex oracle reproduces its committed fixture (regression pin)."""
    z = np.load(os.path.join(GOLDEN, "complex_small.npz"))
    _, _, orc = make_setup(rings=int(z["rings"]), ports=int(z["ports"]), components=int(z["components"]),
                           height=float(z["height"]))
    V, J = oracle.eit_forward_complex(orc, z["gamma"], want_jacobian=True)
    assert np.abs(V - z["V"]).max() / np.abs(z["V"]).max() < 1e-10
    Jp = J @ z["probes"]
    assert np.abs(Jp - z["J_probe"]).max() / np.abs(z["J_probe"]).max() < 1e-9
