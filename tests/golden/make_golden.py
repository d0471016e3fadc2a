"""Regenerates the regression fixtures in this directory from the FP64 oracle.

    python tests/golden/make_golden.py

config1_small.npz: 16-ring disk, 16 electrodes (0.1 rad), adjacent drive
(1 mA) / adjacent measurement, one inclusion (sigma 0.1 in 1.0, r = 0.2,
seeded centre), one harmonic.  Stores the voltages, the Jacobian applied to
four seeded probe vectors, the reference ELL column ids and the port edges.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))          # tests/ (conftest helpers)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from conftest import inclusion_sigma, make_setup  # noqa: E402
import oracle  # noqa: E402


def main():
    rings, ports = 16, 16
    mesh, _, orc = make_setup(rings=rings, ports=ports)
    sigma = inclusion_sigma(mesh, seed=0)
    V, J, _ = oracle.eit_forward(orc, sigma, tol=1e-13)
    probes = np.random.default_rng(123).standard_normal((mesh.elements.shape[0], 4))
    np.savez_compressed(os.path.join(HERE, "config1_small.npz"), rings=rings, ports=ports, sigma=sigma, V=V,
                        J_probe=J @ probes, probes=probes, colIds=orc.layout.colIds, portEdges=orc.portEdges)


if __name__ == "__main__":
    main()
