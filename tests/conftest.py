import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the oracle and the CUDA library once if they are missing or stale."""
    import oracle
    from mpflow_gb300 import build as mbuild
    oracle.build()
    mbuild.build()


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if gpu_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device in this environment")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


def make_setup(rings=16, ports=16, width=0.1, components=1, height=1.0, port_height=1.0, current=1e-3,
               logarithmic=False, ref=1.0):
    """Mesh + adjacent drive/measurement sources for both the library and the oracle."""
    import mpflow_gb300 as mp
    import oracle
    mesh = mp.IrregularMesh.ring(rings)
    pr = mp.Ports.circularBoundary(ports, width, mesh)
    assert (pr.edges >= 0).sum(axis=1).min() >= 1, "mesh too coarse: a port has no boundary edge"
    pat = mp.adjacent_pattern(ports)
    src = mp.Sources(mp.OPEN, current, pr, pat, pat)
    orc = oracle.Setup(mesh.nodes, mesh.elements, mesh.edges, mesh.boundary, pr.edges, pat, pat,
                       np.full(ports, current), ref=ref, logarithmic=logarithmic, components=components,
                       height=height, portHeight=port_height)
    return mesh, src, orc


def inclusion_sigma(mesh, seed=0, background=1.0, value=0.1, radius=0.2, rmax=0.6):
    """Background conductivity with one circular inclusion (seeded centre in r < rmax)."""
    rng = np.random.default_rng(seed)
    r = rmax * np.sqrt(rng.random())
    t = 2 * np.pi * rng.random()
    c = np.array([r * np.cos(t), r * np.sin(t)])
    cent = mesh.nodes[mesh.elements].mean(axis=1)
    g = np.full(mesh.elements.shape[0], background)
    g[np.linalg.norm(cent - c, axis=1) < radius] = value
    return g
