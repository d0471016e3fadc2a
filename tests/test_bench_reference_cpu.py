"""bench.py's reference arm (the FP64 oracle port on the host cores) keeps
the JSON contract: one line with the metric, value, e2e and cpu_baseline
keys, run here on a small mesh; it builds its problem with the oracle alone
and maps none of the library's compiled code."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    args = ["--impl", "reference", "--rings", "16", "--electrodes", "16", "--components", "2", "--steps", "1",
            "--warmup", "0", "--frames", "4"]
    # run bench.py's main in a process that then reports whether the library was mapped
    probe = ("import runpy, sys; sys.argv = ['bench.py'] + sys.argv[1:]; "
             "runpy.run_path('bench.py', run_name='__main__'); "
             "print('LIBMAPPED', 'libmpflow_gb300' in open('/proc/self/maps').read())")
    cmd = [sys.executable, "-c", probe, *args]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["higher_is_better"] is True
    assert line["unit"] == "frames/s" and line["value"] > 0
    for key in ("metric", "n_gpus", "steps", "warmup", "ms_per_step", "scaling", "dtype", "config", "e2e",
                "cpu_baseline"):
        assert key in line, key
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert "LIBMAPPED False" in r.stdout, r.stdout


def test_oracle_ring_mesh_equals_library_mesh():
    """The oracle's ring-mesh generator (used by the reference arm) gives the
    library's mesh bit for bit, so both arms reconstruct the same frames."""
    import numpy as np
    import oracle
    import mpflow_gb300 as mp
    for rings in (1, 2, 7, 30, 80):
        nodes, elements = oracle.ring_mesh(rings)
        mesh = mp.IrregularMesh.ring(rings)
        assert np.array_equal(nodes, mesh.nodes) and np.array_equal(elements, mesh.elements)
        edges, _, boundary = oracle.mesh_edges(nodes, elements)
        assert np.array_equal(edges, mesh.edges) and np.array_equal(boundary, mesh.boundary)
