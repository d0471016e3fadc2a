"""Regenerates the regression fixtures in this directory from the FP64 oracle.

    python tests/golden/make_golden.py

config1_small.npz: 16-ring disk, 16 electrodes (0.1 rad), adjacent drive
(1 mA) / adjacent measurement, one inclusion (sigma 0.1 in 1.0, r = 0.2,
seeded centre), one harmonic.  Stores the voltages, the Jacobian applied to
four seeded probe vectors, the reference ELL column ids and the port edges.

config2_r40.npz: the 2.5D configuration reduced to 40 rings (4921 nodes,
9600 triangles), 32 electrodes, 8 harmonics (height 4), a smooth log-normal
conductivity (exp of 0.5 times a seeded sum of 64 random Fourier features
with wavelengths around 0.15 x 2 pi).  Same contents, two probe vectors.

complex_small.npz: the 16-ring setup with 2 harmonics (height 2) and a
complex admittivity (inclusion conductivity plus an imaginary part); the
complex voltages and the complex Jacobian applied to two complex probes.
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

    # reduced config 2
    mesh, _, orc = make_setup(rings=40, ports=32, width=0.1, components=8, height=4.0)
    cent = mesh.nodes[mesh.elements].mean(axis=1)
    rng = np.random.default_rng(1)
    k = rng.standard_normal((64, 2)) / 0.15
    ph = rng.uniform(0, 2 * np.pi, 64)
    field = np.sqrt(2.0 / 64) * np.cos(cent @ k.T + ph).sum(axis=1)
    sigma = np.exp(0.5 * field)
    V, J, _ = oracle.eit_forward(orc, sigma, tol=1e-13)
    probes = np.random.default_rng(456).standard_normal((mesh.elements.shape[0], 2))
    np.savez_compressed(os.path.join(HERE, "config2_r40.npz"), rings=40, ports=32, components=8, height=4.0,
                        sigma=sigma, V=V, J_probe=J @ probes, probes=probes, colIds=orc.layout.colIds,
                        portEdges=orc.portEdges)

    # complex admittivity
    mesh, _, orc = make_setup(rings=16, ports=16, components=2, height=2.0)
    sig = inclusion_sigma(mesh, seed=3)
    eps = 0.1 + 0.2 * np.random.default_rng(4).random(mesh.elements.shape[0])
    gamma = sig + 1j * eps * sig
    Vz, Jz = oracle.eit_forward_complex(orc, gamma, want_jacobian=True)
    pr = np.random.default_rng(789)
    probes = pr.standard_normal((mesh.elements.shape[0], 2)) + 1j * pr.standard_normal((mesh.elements.shape[0], 2))
    np.savez_compressed(os.path.join(HERE, "complex_small.npz"), rings=16, ports=16, components=2, height=2.0,
                        gamma=gamma, V=Vz, J_probe=Jz @ probes, probes=probes)


if __name__ == "__main__":
    main()
