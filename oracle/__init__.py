"""FP64 CPU oracle for mpFlow's EIT hot path (TEST INFRASTRUCTURE ONLY).

It is the reference results the tests compare against: only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may
import it.  The product library in
``mpflow_gb300`` never imports or links anything here.

The numerical work lives in ``eit_oracle.c`` (an FP64 restatement of the
reference routines, each citing its file:line); this module loads it with
ctypes and composes the reference's forward model and inverse step from it:

* :func:`eit_forward` restates ``EIT::solve`` (src/models/eit.cpp:139-213);
* :func:`inverse_primal` restates ``Inverse::updateJacobian`` + ``solve``
  (src/solver/inverse.cpp:60-238): (J^T J + (ref*lambda)^2 I) dsigma = J^T y;
* :func:`inverse_dual` is the same update in dual form
  J^T (J J^T + mu I)^{-1} y, identical in exact arithmetic for R = I.

Parity status: the reference has no tests or golden vectors and cannot be
built or run here, so this oracle is "parity unpinned"; it is checked by the
known-answer properties in tests/test_oracle.py.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

INVALID = 0xFFFFFFFF
ELL_WIDTH = 32


def build() -> str:
    """Compile eit_oracle.c into oracle/_build/liboracle.so (portable flags)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
                os.path.join(_HERE, "eit_oracle.c")):
            build()
        _lib = ctypes.CDLL(_LIB_PATH)
        _declare(_lib)
    return _lib


_P = ctypes.c_void_p
_I = ctypes.c_int
_U = ctypes.c_uint
_D = ctypes.c_double


def _declare(L):
    L.orc_data_rows.argtypes = [_U]
    L.orc_data_rows.restype = _U
    L.orc_num_threads.restype = _I
    L.orc_set_threads.argtypes = [_I]
    L.orc_ring_mesh.argtypes = [_I, _D, _P, _P]
    L.orc_ring_mesh.restype = _I
    L.orc_mesh_edges.argtypes = [_I, _I, _P, _P, _P, _P, _P, _P]
    L.orc_mesh_edges.restype = _I
    L.orc_circular_ports.argtypes = [_I, _P, _I, _P, _P, _I, _P, _I, _D, _D, _I, _P, _I, _P]
    L.orc_circular_ports.restype = _I
    L.orc_p1_elemental.argtypes = [_I, _P, _P, _P, _P]
    L.orc_equation_levels.argtypes = [_I, _I, _P]
    L.orc_equation_levels.restype = _I
    L.orc_equation_layout.argtypes = [_I, _I, _P, _P, _P, _U, _P, _P, _P, _P, _P]
    L.orc_equation_layout.restype = _I
    L.orc_update_matrix.argtypes = [_U, _U, _P, _P, _P, _D, _I, _P]
    L.orc_update_system_matrix.argtypes = [_U, _P, _P, _P, _U, _D, _P]
    L.orc_excitation_matrix.argtypes = [_I, _P, _P, _I, _P, _I, _P, _I]
    L.orc_ell_multiply.argtypes = [_U, _P, _P, _U, _P, _U, _U, _P]
    L.orc_pcg.argtypes = [_U, _P, _P, _U, _P, _P, _U, _U, _D, _U, _I, _P]
    L.orc_calc_jacobian.argtypes = [_U, _P, _P, _P, _U, _U, _U, _P, _D, _I, _I, _U, _P]
    L.orc_gram_t.argtypes = [_U, _U, _P, _P]
    L.orc_gram_n.argtypes = [_U, _U, _P, _P]
    L.orc_dense_cg.argtypes = [_U, _P, _P, _P, _D, _U]
    L.orc_dense_cg.restype = _U
    L.orc_cholesky.argtypes = [_U, _P]
    L.orc_cholesky.restype = _I
    L.orc_cholesky_solve.argtypes = [_U, _P, _P]


def _p(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def data_rows(n: int) -> int:
    """Padded row count of a reference Matrix (src/numeric/matrix.cpp:49-55)."""
    return int(lib().orc_data_rows(n))


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def num_threads() -> int:
    return int(lib().orc_num_threads())


# --------------------------------------------------------------------------
# mesh, ports, elemental integrals, layout
# --------------------------------------------------------------------------

def mesh_edges(nodes: np.ndarray, elements: np.ndarray):
    """Edge table, element->edge map and boundary list (own convention, see
    orc_mesh_edges)."""
    nodes = np.ascontiguousarray(nodes, dtype=np.float64)
    elements = np.ascontiguousarray(elements, dtype=np.int32)
    N, E = nodes.shape[0], elements.shape[0]
    edges = np.zeros((3 * E, 2), np.int32)
    elementEdges = np.zeros((E, 3), np.int32)
    boundary = np.zeros(3 * E, np.int32)
    nb = ctypes.c_int(0)
    ne = lib().orc_mesh_edges(N, E, _p(nodes), _p(elements), _p(edges), _p(elementEdges),
                              _p(boundary), ctypes.byref(nb))
    if ne < 0:
        raise ValueError("orc_mesh_edges: invalid mesh")
    return edges[:ne].copy(), elementEdges, boundary[:nb.value].copy()


def ring_mesh(rings: int, radius: float = 1.0):
    """Concentric-ring disk (nodes N x 2, elements E x 3) with N = 1 + 3R(R+1)
    and E = 6R^2, the benchmark's mesh; the same numbering as the library's
    generator, written independently (orc_ring_mesh)."""
    R = int(rings)
    nodes = np.zeros((1 + 3 * R * (R + 1), 2))
    elements = np.zeros((6 * R * R, 3), np.int32)
    e = lib().orc_ring_mesh(R, float(radius), _p(nodes), _p(elements))
    if e != elements.shape[0]:
        raise ValueError(f"orc_ring_mesh failed ({e})")
    return nodes, elements


def adjacent_pattern(count: int) -> np.ndarray:
    """Adjacent pattern (+1 on port j, -1 on port j+1), ports x count."""
    p = np.zeros((count, count))
    j = np.arange(count)
    p[j, j] = 1.0
    p[(j + 1) % count, j] = -1.0
    return p


def circular_ports(nodes, elements, edges, boundary, count, width, offset=0.0, clockwise=False,
                   cap=256):
    """Port edge table (count x maxEdges, -1 padded), src/fem/ports.cpp:32-77."""
    nodes = np.ascontiguousarray(nodes, dtype=np.float64)
    elements = np.ascontiguousarray(elements, dtype=np.int32)
    edges = np.ascontiguousarray(edges, dtype=np.int32)
    boundary = np.ascontiguousarray(boundary, dtype=np.int32)
    out = np.full((count, cap), -1, np.int32)
    mx = ctypes.c_int(0)
    st = lib().orc_circular_ports(nodes.shape[0], _p(nodes), elements.shape[0], _p(elements),
                                  _p(edges), boundary.shape[0], _p(boundary), int(count),
                                  float(width), float(offset), int(bool(clockwise)), _p(out), cap,
                                  ctypes.byref(mx))
    if st != 0:
        raise ValueError(f"orc_circular_ports failed with status {st}")
    return out[:, :mx.value].copy()


def p1_elemental(nodes, elements):
    """Per-element 3x3 stiffness K and mass M (src/fem/basis_linear.cpp:72-91)."""
    nodes = np.ascontiguousarray(nodes, dtype=np.float64)
    elements = np.ascontiguousarray(elements, dtype=np.int32)
    E = elements.shape[0]
    K = np.zeros((E, 3, 3))
    M = np.zeros((E, 3, 3))
    lib().orc_p1_elemental(E, _p(nodes), _p(elements), _p(K), _p(M))
    return K, M


@dataclass
class Layout:
    """Reference ELL layout and level decomposition (src/fem/equation.cpp:76-176)."""
    n: int
    dataRows: int
    colIds: np.ndarray          # dataRows x 32 uint32 (row-major, as deviceColumnIds)
    density: int
    levels: int
    connectivity: np.ndarray    # flat, dataRows x (32*levels) column-major
    elemS: np.ndarray           # same layout, float64
    elemR: np.ndarray


def equation_layout(N: int, elements: np.ndarray, K: np.ndarray, M: np.ndarray) -> Layout:
    elements = np.ascontiguousarray(elements, dtype=np.int32)
    E = elements.shape[0]
    levels = lib().orc_equation_levels(N, E, _p(elements))
    if levels < 0:
        raise ValueError("sparse format full")
    dr = data_rows(N)
    colIds = np.zeros((dr, ELL_WIDTH), np.uint32)
    conn = np.zeros(dr * ELL_WIDTH * levels, np.uint32)
    eS = np.zeros(dr * ELL_WIDTH * levels)
    eR = np.zeros(dr * ELL_WIDTH * levels)
    dens = ctypes.c_uint(0)
    K = np.ascontiguousarray(K, dtype=np.float64)
    M = np.ascontiguousarray(M, dtype=np.float64)
    st = lib().orc_equation_layout(N, E, _p(elements), _p(K), _p(M), levels, _p(colIds),
                                   ctypes.byref(dens), _p(conn), _p(eS), _p(eR))
    if st != 0:
        raise ValueError(f"orc_equation_layout failed with status {st}")
    return Layout(N, dr, colIds, int(dens.value), int(levels), conn, eS, eR)


def update_matrix(layout: Layout, elemental: np.ndarray, gamma: np.ndarray, ref: float,
                  logarithmic: bool) -> np.ndarray:
    """ELL values (dataRows x 32), src/fem/equation_kernel.cu:60-82."""
    gamma = np.ascontiguousarray(gamma, dtype=np.float64)
    vals = np.zeros((layout.dataRows, ELL_WIDTH))
    lib().orc_update_matrix(layout.dataRows, layout.levels, _p(layout.connectivity),
                            _p(elemental), _p(gamma), float(ref), int(bool(logarithmic)),
                            _p(vals))
    return vals


def update_system_matrix(layout: Layout, s: np.ndarray, r: np.ndarray, k: float) -> np.ndarray:
    """sys = S + k R on used slots (src/fem/equation_kernel.cu:137-157)."""
    sysv = np.zeros_like(s)
    lib().orc_update_system_matrix(layout.dataRows, _p(s), _p(r), _p(layout.colIds),
                                   layout.density, float(k), _p(sysv))
    return sysv


def excitation_matrix(nodes, edges, portEdges) -> np.ndarray:
    """N x L excitation matrix (src/fem/equation.cpp:183-215)."""
    nodes = np.ascontiguousarray(nodes, dtype=np.float64)
    edges = np.ascontiguousarray(edges, dtype=np.int32)
    portEdges = np.ascontiguousarray(portEdges, dtype=np.int32)
    N = nodes.shape[0]
    L, cap = portEdges.shape
    exc = np.zeros((L, N))   # column-major N x L == row-major L x N
    lib().orc_excitation_matrix(N, _p(nodes), _p(edges), L, _p(portEdges), cap, _p(exc), N)
    return exc.T.copy()


def ell_multiply(layout: Layout, values: np.ndarray, x: np.ndarray) -> np.ndarray:
    """y = A x with x of shape (n, cols) (src/numeric/sparse_matrix_kernel.cu:157-196)."""
    n = layout.n
    xf = np.asfortranarray(x, dtype=np.float64)
    cols = xf.shape[1]
    y = np.zeros((n, cols), order="F")
    lib().orc_ell_multiply(n, _p(values), _p(layout.colIds), layout.density, _p(xf), n, cols,
                           _p(y))
    return y


def pcg(layout: Layout, values: np.ndarray, b: np.ndarray, x0: np.ndarray | None = None,
        tol: float = 1e-12, max_iter: int = 0, dc_free: bool = False):
    """Jacobi-PCG over independent columns (src/numeric/conjugate_gradient.cpp:61-161)."""
    n = layout.n
    bf = np.asfortranarray(b, dtype=np.float64)
    cols = bf.shape[1]
    x = np.zeros((n, cols), order="F") if x0 is None else np.asfortranarray(x0, dtype=np.float64).copy()
    iters = np.zeros(cols, np.uint32)
    lib().orc_pcg(n, _p(values), _p(layout.colIds), layout.density, _p(bf), _p(x), n, cols,
                  float(tol), int(max_iter), int(bool(dc_free)), _p(iters))
    return x, iters


def bicgstab(layout: Layout, values: np.ndarray, b: np.ndarray, x0: np.ndarray | None = None,
             tol: float = 1e-12, max_iter: int = 0):
    """Right-preconditioned BiCGSTAB with the Jacobi preconditioner over
    independent columns, restating BiCGSTAB::solve (src/numeric/bicgstab.cpp:
    83-193): y = K^-1 p, nu = A y, alpha = rho / (rHat, nu), s = r - alpha nu,
    z = K^-1 s, t = A z, omega = (z, K^-1 t) / (K^-1 t, K^-1 t),
    x += alpha y + omega z, r = s - omega t.  The reference stops when column
    0 reaches |r| / |b| < eps; here every column stops on its own at
    |r| <= tol |b| and keeps its x and r from then on.  dcFree is ignored, as
    in the reference.  Returns (x, iterations per column)."""
    n = layout.n
    ids = layout.colIds[:n].astype(np.int64)
    vals = np.asarray(values, np.float64)[:n]
    diag = np.where(ids == np.arange(n)[:, None], vals, 0.0).sum(axis=1)
    dinv = np.where(diag != 0.0, 1.0 / np.where(diag != 0.0, diag, 1.0), 0.0)[:, None]
    b = np.asarray(b, np.float64)
    cols = b.shape[1]
    x = np.zeros((n, cols)) if x0 is None else np.array(x0, np.float64)
    r = b - ell_multiply(layout, values, x)
    rhat = r.copy()
    rho = np.ones(cols)
    alpha = np.ones(cols)
    omega = np.ones(cols)
    nu = np.zeros((n, cols))
    p = np.zeros((n, cols))
    bb = (b * b).sum(axis=0)
    live = (r * r).sum(axis=0) > tol * tol * bb
    iters = np.zeros(cols, np.int64)
    for _ in range(max_iter if max_iter > 0 else 10 * n):
        if not live.any():
            break
        rho_old, rho = rho, np.where(live, (rhat * r).sum(axis=0), rho)
        beta = (rho / rho_old) * (alpha / omega)
        p = np.where(live, r + beta * (p - omega * nu), p)
        y = dinv * p
        nu = np.where(live, ell_multiply(layout, values, y), nu)
        den = (rhat * nu).sum(axis=0)
        alpha = np.where(live, rho / np.where(den != 0.0, den, 1.0), alpha)
        s = r - alpha * nu
        z = dinv * s
        t = ell_multiply(layout, values, z)
        kt = dinv * t
        tt = (kt * kt).sum(axis=0)
        omega = np.where(live, (z * kt).sum(axis=0) / np.where(tt > 0.0, tt, 1.0), omega)
        x = np.where(live, x + alpha * y + omega * z, x)
        r = np.where(live, s - omega * t, r)
        iters += live
        live = live & ((r * r).sum(axis=0) > tol * tol * bb)
    return x, iters


def calc_jacobian(elements, K, phi, drive_count, meas_count, gamma, ref, logarithmic,
                  rowsJ, J=None, additive=False):
    """J (rowsJ x E, column-major), src/fem/equation_kernel.cu:197-245."""
    elements = np.ascontiguousarray(elements, dtype=np.int32)
    E = elements.shape[0]
    phif = np.asfortranarray(phi, dtype=np.float64)
    gamma = np.ascontiguousarray(gamma, dtype=np.float64)
    K = np.ascontiguousarray(K, dtype=np.float64)
    if J is None:
        J = np.zeros((rowsJ, E), order="F")
    lib().orc_calc_jacobian(E, _p(elements), _p(K), _p(phif), phif.shape[0], drive_count,
                            meas_count, _p(gamma), float(ref), int(bool(logarithmic)),
                            int(bool(additive)), rowsJ, _p(J))
    return J


# --------------------------------------------------------------------------
# composed forward model (src/models/eit.cpp)
# --------------------------------------------------------------------------

def _round16(n: int) -> int:
    return ((n + 15) // 16) * 16


def pattern_data_cols(cols: int) -> int:
    """dataCols of a pattern matrix (src/numeric/matrix.cpp:53-55)."""
    return data_rows(cols)


@dataclass
class Setup:
    """Everything EIT::EIT builds once per mesh (src/models/eit.cpp:29-95)."""
    nodes: np.ndarray
    elements: np.ndarray
    edges: np.ndarray
    boundary: np.ndarray
    portEdges: np.ndarray
    drive: np.ndarray            # L x Md
    meas: np.ndarray             # L x Mm
    values: np.ndarray           # Md source values
    ref: float = 1.0
    logarithmic: bool = False
    components: int = 1
    height: float = 1.0
    portHeight: float = 1.0
    K: np.ndarray = field(default=None)
    M: np.ndarray = field(default=None)
    layout: Layout = field(default=None)
    exc: np.ndarray = field(default=None)

    def __post_init__(self):
        self.K, self.M = p1_elemental(self.nodes, self.elements)
        self.layout = equation_layout(self.nodes.shape[0], self.elements, self.K, self.M)
        self.exc = excitation_matrix(self.nodes, self.edges, self.portEdges)

    @property
    def Md(self):
        return self.drive.shape[1]

    @property
    def Mm(self):
        return self.meas.shape[1]

    @property
    def rowsJ(self):
        return pattern_data_cols(self.Mm) * pattern_data_cols(self.Md)

    def alpha_beta(self, c: int):
        """2.5D constants of component c (src/models/eit.cpp:154-157)."""
        alpha = (2.0 * c * math.pi / self.height) ** 2
        beta = (1.0 / self.height) if c == 0 else (
            2.0 * math.sin(c * math.pi * self.portHeight / self.height) /
            (c * math.pi * self.portHeight))
        return alpha, beta


def eit_forward(s: Setup, gamma: np.ndarray, tol: float = 1e-12, want_jacobian: bool = True,
                max_iter: int = 0, exact: bool = False, solver: str = "cg"):
    """Restatement of EIT::solve for current (Open) sources (solver "cg" or
    "bicgstab", the numericalSolverType template argument of models::EIT).

    Returns (V, J, fields): V is Mm x Md, J is rowsJ x E column-major (row =
    drive * roundMeas + meas), fields is a list of n x (Md+Mm) arrays per
    component.  exact=True replaces the reference's 2.5D Jacobian (stiffness
    term only, weight height*beta_c^2) by the exact derivative of V (element
    matrix K + alpha_c M, weight beta_c); both agree for one harmonic."""
    n = s.nodes.shape[0]
    pattern = np.concatenate([s.drive * s.values[None, :], s.meas], axis=1)
    att = (s.meas.T @ s.exc.T)                       # Mm x N  (eit.cpp:93-94)
    S = update_matrix(s.layout, s.layout.elemS, gamma, s.ref, s.logarithmic)
    R = update_matrix(s.layout, s.layout.elemR, gamma, s.ref, s.logarithmic)
    V = np.zeros((s.Mm, s.Md))
    J = np.zeros((s.rowsJ, s.elements.shape[0]), order="F") if want_jacobian else None
    fields = []
    for c in range(s.components):
        alpha, beta = s.alpha_beta(c)
        sysv = update_system_matrix(s.layout, S, R, alpha)
        excitation = (s.exc @ pattern) * beta
        if solver == "bicgstab":
            x, _ = bicgstab(s.layout, sysv, excitation, tol=tol, max_iter=max_iter)
        else:
            x, _ = pcg(s.layout, sysv, excitation, tol=tol, max_iter=max_iter, dc_free=(c == 0))
        fields.append(x)
        if want_jacobian and not exact:
            calc_jacobian(s.elements, s.K, x, s.Md, s.Mm, gamma, s.ref, s.logarithmic, s.rowsJ,
                          J=J, additive=(c > 0))
        elif want_jacobian and abs(beta) > 1e-12 / s.height:
            Jc = calc_jacobian(s.elements, s.K + alpha * s.M, x, s.Md, s.Mm, gamma, s.ref,
                               s.logarithmic, s.rowsJ)
            J += Jc / (beta * s.height)
        V += att @ x[:, :s.Md]
    if want_jacobian:
        J *= s.height
        J *= -1.0
    return V, J, fields


def flatten_measurement(V: np.ndarray, s: Setup) -> np.ndarray:
    """Column-major flattening of an Mm x Md voltage matrix with padded rows,
    the order Inverse::calcExcitation reads it in (src/solver/inverse.cpp:163-205)."""
    mp = pattern_data_cols(s.Mm)
    out = np.zeros((mp, pattern_data_cols(s.Md)))
    out[:s.Mm, :s.Md] = V
    return out.reshape(-1, order="F")


def inverse_primal(J: np.ndarray, y: np.ndarray, ref: float, lam: float, tol: float = 1e-14):
    """(J^T J + (ref*lam)^2 I) dsigma = J^T y by dense CG (src/solver/inverse.cpp:60-238)."""
    rows, E = J.shape
    Jf = np.asfortranarray(J, dtype=np.float64)
    G = np.zeros((E, E), order="F")
    lib().orc_gram_t(rows, E, _p(Jf), _p(G))
    G[np.diag_indices(E)] += (ref * lam) ** 2
    g = Jf.T @ y
    x = np.zeros(E)
    lib().orc_dense_cg(E, _p(G), _p(np.ascontiguousarray(g)), _p(x), float(tol), 0)
    return x


def inverse_dual(J: np.ndarray, y: np.ndarray, ref: float, lam: float) -> np.ndarray:
    """Same update in dual form J^T (J J^T + mu I)^{-1} y via FP64 Cholesky."""
    rows, E = J.shape
    Jf = np.asfortranarray(J, dtype=np.float64)
    G = np.zeros((rows, rows), order="F")
    lib().orc_gram_n(rows, E, _p(Jf), _p(G))
    G[np.diag_indices(rows)] += (ref * lam) ** 2
    info = lib().orc_cholesky(rows, _p(G))
    if info != 0:
        raise np.linalg.LinAlgError(f"Cholesky failed at pivot {info}")
    w = np.ascontiguousarray(y, dtype=np.float64).copy()
    lib().orc_cholesky_solve(rows, _p(G), _p(w))
    return Jf.T @ w


def laplacian_gram(nodes: np.ndarray, elements: np.ndarray) -> np.ndarray:
    """L^T L of the edge-length Laplacian of Inverse::calcRegularizationMatrix
    (src/solver/inverse.cpp:98-113): L[edge][element] = sign * |edge| with the
    sign flipping between the two elements that share an edge (dense E x E)."""
    E = elements.shape[0]
    LtL = np.zeros((E, E))
    first = {}
    for e in range(E):
        for i in range(3):
            a, b = int(elements[e, i]), int(elements[e, (i + 1) % 3])
            key = (min(a, b), max(a, b))
            l2 = float(((nodes[a] - nodes[b]) ** 2).sum())
            LtL[e, e] += l2
            if key in first:
                o = first[key]
                LtL[e, o] -= l2
                LtL[o, e] -= l2
            else:
                first[key] = e
    return LtL


def inverse_regularised(J: np.ndarray, Y: np.ndarray, ref: float, factor: float, kind: str,
                        nodes=None, elements=None) -> np.ndarray:
    """(J^T J + (ref*factor)^2 R) X = J^T Y in FP64 for R = I, diag(J^T J)
    (NOSER) or the Laplacian L^T L (src/solver/inverse.cpp:60-130,213-238),
    solved directly.  J: rows x E, Y: rows x images; returns E x images.
    Complex J and Y (the thrust::complex instantiations) use the plain
    transpose, as the reference's CUBLAS_OP_T products."""
    JtJ = J.T @ J
    mu = (ref * factor) ** 2
    if kind == "identity":
        R = np.eye(J.shape[1])
    elif kind == "noser":
        R = np.diag(np.diag(JtJ))
    elif kind == "laplacian":
        R = laplacian_gram(nodes, elements)
    else:
        raise ValueError(kind)
    return np.linalg.solve(JtJ + mu * R, J.T @ Y)


def dense_matrix(layout: Layout, values: np.ndarray, n: int) -> np.ndarray:
    """Dense n x n matrix of reference-ELL slot values (rows x 32)."""
    A = np.zeros((n, n))
    ids = layout.colIds[:n]
    v = values[:n]
    rows, ks = np.nonzero(ids != INVALID)
    np.add.at(A, (rows, ids[rows, ks].astype(np.int64)), v[rows, ks])
    return A


def eit_forward_fixed(s: Setup, gamma: np.ndarray, want_jacobian: bool = True):
    """Restatement of EIT::solve for voltage (Fixed) sources
    (src/models/eit.cpp:85-91,160-205,251-270, src/models/eit_kernel.cu:34-54):
    the excitation matrix is binarised (|Exc| >= 1e-9 -> 1), every node that
    belongs to a port gets a Dirichlet row (identity) carrying the port's
    voltage, the harmonics are not weighted by beta, the measured quantity is
    the current height * A x collected by the binarised attachment matrix,
    and J = +height * sum_c J_c.  Solved exactly (dense), which is the limit
    the reference's CG converges to."""
    n = s.nodes.shape[0]
    excb = (np.abs(s.exc) >= 1e-9).astype(np.float64)
    dirichlet = excb.any(axis=1)
    pattern = np.concatenate([s.drive * s.values[None, :], s.meas], axis=1)
    att = s.meas.T @ excb.T
    S = dense_matrix(s.layout, update_matrix(s.layout, s.layout.elemS, gamma, s.ref, s.logarithmic), n)
    R = dense_matrix(s.layout, update_matrix(s.layout, s.layout.elemR, gamma, s.ref, s.logarithmic), n)
    V = np.zeros((s.Mm, s.Md))
    J = np.zeros((s.rowsJ, s.elements.shape[0]), order="F") if want_jacobian else None
    fields = []
    for c in range(s.components):
        alpha, _ = s.alpha_beta(c)
        A = S + alpha * R
        Ab = A.copy()
        Ab[dirichlet, :] = 0.0
        Ab[dirichlet, dirichlet] = 1.0
        x = np.linalg.solve(Ab, excb @ pattern)
        fields.append(x)
        if want_jacobian:
            calc_jacobian(s.elements, s.K, x, s.Md, s.Mm, gamma, s.ref, s.logarithmic, s.rowsJ,
                          J=J, additive=(c > 0))
        V += att @ (s.height * (A @ x))[:, :s.Md]
    if want_jacobian:
        J *= s.height
    return V, J, fields


def calc_jacobian_complex(s: Setup, phi: np.ndarray, gamma: np.ndarray) -> np.ndarray:
    """calcJacobianKernel (src/fem/equation_kernel.cu:197-245) for complex
    fields phi (n x (Md+Mm)) and complex gamma: rowsJ x E, row
    d * roundMeas + m, J[row, e] = p'(gamma_e) sum_ij phi[n_i, d] K_e[i + 3 j]
    phi[n_j, Md + m] (bilinear, no conjugation)."""
    E = s.elements.shape[0]
    g = np.asarray(gamma, np.complex128)
    deriv = s.ref * (math.log(10.0) / 10.0) * np.exp(math.log(10.0) * g / 10.0) if s.logarithmic else \
        np.full(E, s.ref, np.complex128)
    Kr = np.asarray(s.K, np.float64).reshape(E, 3, 3)        # flat i + 3 j -> Kr[e, j, i]
    nodes = phi[s.elements]                                  # E x 3 x (Md+Mm)
    el = np.einsum("eid,eji,ejm->edm", nodes[:, :, :s.Md], Kr, nodes[:, :, s.Md:s.Md + s.Mm])
    roundMeas = _round16(s.Mm)
    J = np.zeros((s.rowsJ, E), np.complex128)
    for d in range(s.Md):
        J[d * roundMeas:d * roundMeas + s.Mm, :] = (el[:, d, :] * deriv[:, None]).T
    return J


def eit_forward_complex(s: Setup, gamma: np.ndarray, want_jacobian: bool = False, want_fields: bool = False):
    """Restatement of EIT::solve for complex material values (the
    Equation<thrust::complex<T>> instantiations, src/models/eit.cpp:139-245
    and :289-304; p(gamma) of src/fem/equation_kernel.cu:35-43 with complex
    gamma), current sources.  The complex systems are solved directly in FP64
    (the reference iterates to the same solution); the Neumann harmonic is
    (A + 1 1^T) x = b as in the reference's CG.  Returns V (Mm x Md, complex)
    and, with want_jacobian, (V, J) with J = -h sum_c J_c (rowsJ x E); with
    want_fields the list of n x (Md + Mm) complex fields per component is
    appended to the returned tuple."""
    g = np.asarray(gamma, np.complex128)
    p = s.ref * (np.exp(math.log(10.0) * g / 10.0) if s.logarithmic else g)
    S = (update_matrix(s.layout, s.layout.elemS, p.real, 1.0, False) +
         1j * update_matrix(s.layout, s.layout.elemS, p.imag, 1.0, False))
    R = (update_matrix(s.layout, s.layout.elemR, p.real, 1.0, False) +
         1j * update_matrix(s.layout, s.layout.elemR, p.imag, 1.0, False))
    n = s.nodes.shape[0]
    pattern = np.concatenate([s.drive * s.values[None, :], s.meas], axis=1)
    att = s.meas.T @ s.exc.T
    V = np.zeros((s.Mm, s.Md), np.complex128)
    J = np.zeros((s.rowsJ, s.elements.shape[0]), np.complex128) if want_jacobian else None
    fields = []
    for c in range(s.components):
        alpha, beta = s.alpha_beta(c)
        sys_re = update_system_matrix(s.layout, S.real.copy(), R.real.copy(), alpha)
        sys_im = update_system_matrix(s.layout, S.imag.copy(), R.imag.copy(), alpha)
        A = dense_matrix(s.layout, sys_re, n) + 1j * dense_matrix(s.layout, sys_im, n)
        if c == 0:
            A = A + 1.0
        x = np.linalg.solve(A, (s.exc @ pattern) * beta)
        fields.append(x)
        V += att @ x[:, :s.Md]
        if want_jacobian:
            J += calc_jacobian_complex(s, x, g)
    out = (V, -s.height * J) if want_jacobian else (V,)
    if want_fields:
        out = out + (fields,)
    return out if len(out) > 1 else out[0]
