"""Known-answer tests of the complete-electrode-model oracle (oracle/cem.py),
which has no reference counterpart: reciprocity, current conservation at the
electrodes, its Jacobian against central finite differences, and the
z -> 0 limit, the shunt model of perfectly conducting electrodes."""
import numpy as np
import pytest

from conftest import inclusion_sigma


def _setup(rings=20, ports=16, components=2, height=2.0, logarithmic=True):
    import oracle
    nodes, elements = oracle.ring_mesh(rings)
    edges, _, boundary = oracle.mesh_edges(nodes, elements)
    ports_e = oracle.circular_ports(nodes, elements, edges, boundary, ports, 0.1)
    assert (ports_e >= 0).sum(axis=1).min() >= 1, "mesh too coarse: a port has no boundary edge"
    pat = oracle.adjacent_pattern(ports)
    s = oracle.Setup(nodes, elements, edges, boundary, ports_e, pat, pat, np.full(ports, 1e-3), ref=1.0,
                     logarithmic=logarithmic, components=components, height=height)
    return s


def _gamma(s, seed=2):
    class M:  # inclusion_sigma only needs nodes and elements
        nodes, elements = s.nodes, s.elements
    return 10 * np.log10(inclusion_sigma(M, seed=seed, value=0.3))


def test_cem_voltages_are_reciprocal():
    from oracle.cem import eit_forward_cem
    s = _setup()
    V, _, _ = eit_forward_cem(s, _gamma(s), 1e-2, want_jacobian=False)
    assert np.abs(V - V.T).max() <= 1e-10 * np.abs(V).max()


def test_cem_electrode_currents_are_the_injected_ones():
    from oracle.cem import eit_forward_cem, electrode_currents
    s = _setup()
    g = _gamma(s)
    _, _, fields = eit_forward_cem(s, g, 1e-2, want_jacobian=False)
    pattern = np.concatenate([s.drive * s.values[None, :], s.meas], axis=1)
    for c in range(s.components):
        _, beta = s.alpha_beta(c)
        I = electrode_currents(s, g, 1e-2, fields[c])
        # every electrode carries its pattern current; their sum is zero
        assert np.abs(I - beta * pattern).max() <= 1e-9 * np.abs(beta * pattern).max()
        assert np.abs(I.sum(axis=0)).max() <= 1e-9 * np.abs(I).max()


@pytest.mark.parametrize("exact", [True])
def test_cem_jacobian_matches_finite_differences(exact):
    import oracle
    from oracle.cem import eit_forward_cem
    s = _setup(rings=20)
    g = _gamma(s)
    z = 1e-2
    V, J, _ = eit_forward_cem(s, g, z, exact=exact)
    rng = np.random.default_rng(4)
    d = rng.standard_normal(g.size)
    h = 1e-4
    Vp, _, _ = eit_forward_cem(s, g + h * d, z, want_jacobian=False)
    Vm, _, _ = eit_forward_cem(s, g - h * d, z, want_jacobian=False)
    fd = oracle.flatten_measurement((Vp - Vm) / (2 * h), s)
    lin = J @ d
    assert np.abs(lin - fd).max() <= 1e-5 * np.abs(fd).max(), np.abs(lin - fd).max() / np.abs(fd).max()


def test_cem_tends_to_the_shunt_model_as_z_vanishes():
    from oracle.cem import eit_forward_cem, eit_forward_shunt
    s = _setup(rings=24, components=1)
    g = _gamma(s)
    Vs = eit_forward_shunt(s, g)
    errs = []
    for z in (1e-1, 1e-2, 1e-3, 1e-4, 1e-5):
        V, _, _ = eit_forward_cem(s, g, z, want_jacobian=False)
        errs.append(np.abs(V - Vs).max() / np.abs(Vs).max())
    assert all(b < a for a, b in zip(errs, errs[1:])), errs
    assert errs[-1] < 1e-3, errs
