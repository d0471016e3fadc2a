"""Host-side setup of the library (no GPU) against the oracle: mesh topology,
ports, ELL layout and element integrals must agree bit for bit (indices) or
to FP64 rounding (values)."""
import ctypes

import numpy as np
import pytest

import mpflow_gb300 as mp
import oracle
from mpflow_gb300._ffi import lib, ptr


@pytest.mark.parametrize("rings", [1, 2, 7, 30])
def test_ring_mesh_is_valid(rings):
    mesh = mp.IrregularMesh.ring(rings)
    N, E = mesh.nodes.shape[0], mesh.elements.shape[0]
    assert N == 1 + 3 * rings * (rings + 1) and E == 6 * rings * rings
    p = mesh.nodes[mesh.elements]
    det = (p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1]) - (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1])
    assert det.min() > 0  # counter-clockwise, non-degenerate
    # conforming: total area is the inscribed 6R-gon, boundary has 6R edges
    assert abs(0.5 * det.sum() - 0.5 * 6 * rings * np.sin(2 * np.pi / (6 * rings))) < 1e-12
    assert mesh.boundary.shape[0] == 6 * rings
    assert mesh.edges.shape[0] == N + E - 1


@pytest.mark.parametrize("rings", [3, 16, 40])
def test_edges_match_oracle(rings):
    mesh = mp.IrregularMesh.ring(rings)
    e, ee, b = oracle.mesh_edges(mesh.nodes, mesh.elements)
    assert np.array_equal(e, mesh.edges)
    assert np.array_equal(ee, mesh.elementEdges)
    assert np.array_equal(b, mesh.boundary)


@pytest.mark.parametrize("count,width,offset,clockwise", [(16, 0.1, 0.0, False), (32, 0.1, 0.0, False),
                                                         (16, 0.25, 0.3, True), (8, 0.5, -0.2, False)])
def test_ports_match_oracle(count, width, offset, clockwise):
    mesh = mp.IrregularMesh.ring(40)
    ports = mp.Ports.circularBoundary(count, width, mesh, offset, clockwise)
    po = oracle.circular_ports(mesh.nodes, mesh.elements, mesh.edges, mesh.boundary, count, width, offset,
                               clockwise)
    assert np.array_equal(ports.edges, po)
    # every port edge lies on the boundary, edges of a port are distinct
    for row in ports.edges:
        row = row[row >= 0]
        assert len(row) > 0 and set(row.tolist()) <= set(mesh.boundary.tolist())


def test_ell_layout_matches_oracle():
    mesh = mp.IrregularMesh.ring(25)
    N, E = mesh.nodes.shape[0], mesh.elements.shape[0]
    K, M = oracle.p1_elemental(mesh.nodes, mesh.elements)
    lay = oracle.equation_layout(N, mesh.elements, K, M)
    ids = np.zeros((oracle.data_rows(N), 32), np.uint32)
    dens = ctypes.c_uint32(0)
    assert lib().mpf_ell_layout(N, E, ptr(mesh.elements), ptr(ids), ctypes.byref(dens)) == 0
    assert np.array_equal(ids, lay.colIds)
    assert dens.value == lay.density


def test_p1_integrals_match_oracle():
    mesh = mp.IrregularMesh.ring(20)
    E = mesh.elements.shape[0]
    K = np.zeros((E, 3, 3))
    M = np.zeros((E, 3, 3))
    assert lib().mpf_p1_elemental(E, ptr(mesh.nodes), ptr(mesh.elements), ptr(K), ptr(M)) == 0
    Ko, Mo = oracle.p1_elemental(mesh.nodes, mesh.elements)
    assert np.abs(K - Ko).max() / np.abs(Ko).max() < 1e-13
    assert np.abs(M - Mo).max() / np.abs(Mo).max() < 1e-14


def test_excitation_matrix_matches_oracle():
    mesh = mp.IrregularMesh.ring(30)
    ports = mp.Ports.circularBoundary(16, 0.1, mesh)
    N = mesh.nodes.shape[0]
    exc = np.zeros((16, N))
    assert lib().mpf_excitation_matrix(N, ptr(mesh.nodes), ptr(mesh.edges), 16, ptr(ports.edges),
                                       ports.edges.shape[1], ptr(exc), N) == 0
    eo = oracle.excitation_matrix(mesh.nodes, mesh.edges, ports.edges)
    assert np.abs(exc.T - eo).max() < 1e-15
    # every port column integrates the unit current density to one
    assert np.abs(exc.sum(axis=1) - 1).max() < 1e-14


def test_sparse_format_full_is_reported():
    # a fan of 40 triangles around node 0 gives node 0 more than 32 neighbours
    k = 40
    ang = np.linspace(0, 2 * np.pi, k, endpoint=False)
    nodes = np.vstack([[0, 0], np.c_[np.cos(ang), np.sin(ang)]])
    elements = np.array([[0, 1 + i, 1 + (i + 1) % k] for i in range(k)], np.int32)
    ids = np.zeros((oracle.data_rows(k + 1), 32), np.uint32)
    dens = ctypes.c_uint32(0)
    st = lib().mpf_ell_layout(k + 1, k, ptr(elements), ptr(ids), ctypes.byref(dens))
    assert st == 7  # MPF_EFULL, the reference's "sparse format full"
    assert b"sparse format full" in lib().mpf_last_error()
