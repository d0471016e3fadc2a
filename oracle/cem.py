"""FP64 oracle of the complete electrode model (test infrastructure only).

The reference has no electrode model beyond its gap model (a port is a set of
boundary edges, src/fem/ports.cpp:32-77, src/fem/equation.cpp:183-215).  The
complete electrode model is written here from Somersalo, Cheney and Isaacson,
"Existence and uniqueness for electrode models for electric current computed
tomography", SIAM J. Appl. Math. 52 (1992) 1023-1040:

    div(sigma grad u) = 0 in the domain,
    u + z sigma du/dn = U_l on electrode e_l,  sigma du/dn = 0 off the electrodes,
    int_{e_l} sigma du/dn ds = I_l,

whose P1 weak form has the node potentials u and the electrode voltages U as
unknowns:

    [ K(sigma) + C      -B     ] [u]   [0]
    [ -B^T          diag(|e|/z)] [U] = [I],

C = (1/z) int_e phi_i phi_j ds, B = (1/z) int_{e_l} phi_i ds.  The 2.5D model
of the library (src/models/eit.cpp:139-213: harmonics c with alpha_c =
(2 pi c / height)^2, the excitation weighted by beta_c) carries the same
contact term in every harmonic; the voltages are the electrode unknowns,
summed over harmonics like the gap model's port means.  Each harmonic is
solved exactly with a sparse LU (scipy); the Neumann harmonic is grounded at
the last electrode (the voltages are differences of electrode voltages).
"""
from __future__ import annotations

import numpy as np

from . import calc_jacobian


def _mat_param(ref: float, v: np.ndarray, logarithmic: bool) -> np.ndarray:
    # src/fem/equation_kernel.cu:35-43
    return ref * np.power(10.0, v / 10.0) if logarithmic else ref * v


def contact_terms(nodes, edges, port_edges, z: float):
    """(C, B, D) of the contact impedance: C (N x N, sparse), B (N x L,
    sparse) and D (L) with D_l = |e_l| / z, from the port edge table."""
    import scipy.sparse as sp
    N, L = nodes.shape[0], port_edges.shape[0]
    ri, ci, cv, bi, bl, bv = [], [], [], [], [], []
    D = np.zeros(L)
    for l in range(L):
        for eg in port_edges[l]:
            if eg < 0:
                continue
            a, b = int(edges[eg, 0]), int(edges[eg, 1])
            h = float(np.hypot(*(nodes[a] - nodes[b])))
            for (i, j, v) in ((a, a, h / 3), (b, b, h / 3), (a, b, h / 6), (b, a, h / 6)):
                ri.append(i)
                ci.append(j)
                cv.append(v / z)
            for i in (a, b):
                bi.append(i)
                bl.append(l)
                bv.append(h / 2 / z)
            D[l] += h / z
    C = sp.coo_matrix((cv, (ri, ci)), shape=(N, N)).tocsr()
    B = sp.coo_matrix((bv, (bi, bl)), shape=(N, L)).tocsr()
    return C, B, D


def _assemble(s, elemental, sigma):
    import scipy.sparse as sp
    el = s.elements
    rows = np.repeat(el, 3, axis=1).reshape(-1)
    cols = np.tile(el, (1, 3)).reshape(-1)
    E = el.shape[0]
    vals = (np.asarray(elemental, np.float64).reshape(E, 9) * sigma[:, None]).reshape(-1)  # symmetric 3 x 3
    N = s.nodes.shape[0]
    return sp.coo_matrix((vals, (rows, cols)), shape=(N, N)).tocsr()


def cem_system(s, gamma: np.ndarray, z: float, c: int):
    """The complete-electrode system matrix of harmonic c, (N + L) x (N + L)."""
    import scipy.sparse as sp
    sigma = _mat_param(s.ref, np.asarray(gamma, np.float64), s.logarithmic)
    K = _assemble(s, s.K, sigma)
    Mm = _assemble(s, s.M, sigma)
    C, B, D = contact_terms(s.nodes, s.edges, s.portEdges, z)
    alpha, _ = s.alpha_beta(c)
    top = sp.hstack([K + alpha * Mm + C, -B])
    bottom = sp.hstack([-B.T, sp.diags(D)])
    return sp.vstack([top, bottom]).tocsc()


def _solve(A, rhs, ground: bool):
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    if ground:
        # U_{L-1} = 0: the Neumann system determines the potentials up to a constant
        n = A.shape[0]
        keep = np.ones(n, bool)
        keep[-1] = False
        x = np.zeros_like(rhs)
        lu = sla.splu(sp.csc_matrix(A[keep][:, keep]))
        x[keep] = lu.solve(np.ascontiguousarray(rhs[keep]))
        return x
    return sla.splu(A).solve(np.ascontiguousarray(rhs))


def eit_forward_cem(s, gamma: np.ndarray, z: float, want_jacobian: bool = True, exact: bool = True):
    """V (Mm x Md), J (rowsJ x E column-major, the library's row order) and
    the fields per harmonic ((N + L) x (Md + Mm)) of the complete electrode
    model with contact impedance z on every port (Setup s of the oracle:
    mesh, ports, patterns, 2.5D constants).  exact=True: J is the derivative
    of V (element matrix K + alpha_c M, weight beta_c); exact=False: the
    reference's 2.5D formula (stiffness term, weight height beta_c^2)."""
    N, L = s.nodes.shape[0], s.portEdges.shape[0]
    gamma = np.asarray(gamma, np.float64)
    pattern = np.concatenate([s.drive * s.values[None, :], s.meas], axis=1)  # L x (Md + Mm)
    V = np.zeros((s.Mm, s.Md))
    J = np.zeros((s.rowsJ, s.elements.shape[0]), order="F") if want_jacobian else None
    fields = []
    for c in range(s.components):
        alpha, beta = s.alpha_beta(c)
        A = cem_system(s, gamma, z, c)
        rhs = np.zeros((N + L, pattern.shape[1]))
        rhs[N:] = pattern * beta
        x = _solve(A, rhs, ground=(c == 0))
        fields.append(x)
        if want_jacobian and not exact:
            calc_jacobian(s.elements, s.K, np.ascontiguousarray(x[:N]), s.Md, s.Mm, gamma, s.ref, s.logarithmic,
                          s.rowsJ, J=J, additive=(c > 0))
        elif want_jacobian and abs(beta) > 1e-12 / s.height:
            Jc = calc_jacobian(s.elements, s.K + alpha * s.M, np.ascontiguousarray(x[:N]), s.Md, s.Mm, gamma,
                               s.ref, s.logarithmic, s.rowsJ)
            J += Jc / (beta * s.height)
        V += s.meas.T @ x[N:, :s.Md]
    if want_jacobian:
        J *= s.height
        J *= -1.0
    return V, J, fields


def electrode_currents(s, gamma: np.ndarray, z: float, fields_c: np.ndarray) -> np.ndarray:
    """Currents through the electrodes, (1/z) int_{e_l} (U_l - u) ds, of the
    fields of one harmonic (L x columns)."""
    N = s.nodes.shape[0]
    C, B, D = contact_terms(s.nodes, s.edges, s.portEdges, z)
    u, U = fields_c[:N], fields_c[N:]
    return D[:, None] * U - B.T @ u


def eit_forward_shunt(s, gamma: np.ndarray):
    """Voltages (Mm x Md) of the shunt model, the complete electrode model's
    z -> 0 limit: every electrode is a perfect conductor, so the nodes of a
    port share one potential U_l and the port current enters it."""
    import scipy.sparse as sp
    N, L = s.nodes.shape[0], s.portEdges.shape[0]
    owner = np.full(N, -1)
    for l in range(L):
        for eg in s.portEdges[l]:
            if eg >= 0:
                owner[s.edges[eg]] = l
    free = np.flatnonzero(owner < 0)
    idx = np.empty(N, np.int64)
    idx[free] = np.arange(free.size)
    idx[owner >= 0] = free.size + owner[owner >= 0]
    P = sp.coo_matrix((np.ones(N), (np.arange(N), idx)), shape=(N, free.size + L)).tocsr()
    sigma = _mat_param(s.ref, np.asarray(gamma, np.float64), s.logarithmic)
    pattern = np.concatenate([s.drive * s.values[None, :], s.meas], axis=1)
    V = np.zeros((s.Mm, s.Md))
    for c in range(s.components):
        alpha, beta = s.alpha_beta(c)
        A = (P.T @ (_assemble(s, s.K, sigma) + alpha * _assemble(s, s.M, sigma)) @ P).tocsc()
        rhs = np.zeros((free.size + L, pattern.shape[1]))
        rhs[free.size:] = pattern * beta
        x = _solve(A, rhs, ground=(c == 0))
        V += s.meas.T @ x[free.size:, :s.Md]
    return V
