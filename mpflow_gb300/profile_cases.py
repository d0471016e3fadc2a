"""Single-kernel cases for profiling, at the bench workload's shapes.

    python -m mpflow_gb300.profile_cases fem --frames 4
        assembly (k_assemble) and Jacobian (k_jacobian) of F frames of the
        80-ring, 32-electrode, 8-harmonic model (log conductivity, 1-3
        inclusions), timed with CUDA events (mpf_eit_profile_fem);
    python -m mpflow_gb300.profile_cases gn --frames 4 [--gn-factor fp32-refined]
        Gauss-Newton steps from the homogeneous start on F frames of that
        model (split-BF16 Gram, FP64 Cholesky k_potrf_diag / k_trsm / k_syrk
        and triangular solves k_chol_solve, or the FP32 factor with FP64
        refinement), with the device time per phase;
    python -m mpflow_gb300.profile_cases mlp --steps 20
        training steps (mpf_mlp_train_step) of the 1024-2048-2048-38400
        network on batches of 256 rows gathered from 16384 pairs, timed with
        CUDA events.

Each prints one JSON line.  Small enough for a profiler to replay (a few GB
on the device at most)."""
from __future__ import annotations

import argparse
import json

import numpy as np


def _model(mp):
    mesh = mp.IrregularMesh.ring(80)
    ports = mp.Ports.circularBoundary(32, 0.1, mesh)
    pat = mp.adjacent_pattern(32)
    src = mp.Sources(mp.OPEN, 1e-3, ports, pat, pat)
    model = mp.EIT(mesh, src, 1.0, components=8, height=4.0, logarithmic=True, exact_jacobian=True)
    return mesh, model


def case_fem(frames: int, reps: int) -> dict:
    import torch
    import mpflow_gb300 as mp
    from mpflow_gb300.learned import inclusion_frames
    mesh, model = _model(mp)
    cent = mesh.nodes[mesh.elements].mean(axis=1)
    g = torch.tensor(inclusion_frames(cent, frames, np.random.default_rng(7)), device="cuda")
    ms, by = model.profile_fem(g, reps=reps)
    return {"case": "fem", "frames": frames, "k_assemble_ms": float(ms[0]), "k_jacobian_ms": float(ms[1]),
            "k_assemble_gbs": float(by[0] / ms[0] / 1e6), "k_jacobian_gbs": float(by[1] / ms[1] / 1e6),
            "algorithmic_bytes": [float(by[0]), float(by[1])]}


def case_gn(frames: int, gn_factor: str, reps: int) -> dict:
    import torch
    import mpflow_gb300 as mp
    from mpflow_gb300.learned import inclusion_frames
    mesh, model = _model(mp)
    E = mesh.elements.shape[0]
    cent = mesh.nodes[mesh.elements].mean(axis=1)
    vt = torch.tensor(inclusion_frames(cent, frames, np.random.default_rng(3)), device="cuda")
    Vm = model.solve(vt, mp.SolveOptions(tol=1e-6, refine_tol=1e-9)).contiguous()
    _, J0 = model.solve(torch.zeros((1, E), device="cuda"), mp.SolveOptions(tol=1e-6), jacobian=True)
    lam = 2e-2 * float(J0.norm() / np.sqrt(J0.shape[1]))
    opts = mp.SolveOptions(tol=1e-5, gn_factor=gn_factor)
    g = torch.zeros((frames, E), device="cuda")
    res = model.gn_step(g, Vm, lam, opts)  # first step: autotuning and buffers
    phases = {}
    for _ in range(reps):
        g = torch.zeros((frames, E), device="cuda")
        model.phase_times(True)
        res = model.gn_step(g, Vm, lam, opts)
        ph, _ = model.phase_times(False)
        for k, v in ph.items():
            phases[k] = phases.get(k, 0.0) + v / reps
    return {"case": "gn", "frames": frames, "gn_factor": gn_factor,
            "residuals": [float(r) for r in np.asarray(res).ravel()][:8],
            "phase_ms": {k: round(v, 3) for k, v in phases.items() if v > 0}}


def case_mlp(steps: int) -> dict:
    import torch
    import mpflow_gb300 as mp
    net = mp.MLP(1024, 2048, 2048, 38400, seed=1)
    X = torch.randn((16384, 1024), device="cuda")
    T = torch.randn((16384, 38400), device="cuda")
    perm = torch.randperm(16384, device="cuda").to(torch.int32)
    batches = [perm[(i * 256) % 16384:(i * 256) % 16384 + 256] for i in range(steps + 3)]
    for rows in batches[:3]:
        net.train_step(X, T, rows=rows, valid=38400, lr=1e-3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for rows in batches[3:]:
        net.train_step(X, T, rows=rows, valid=38400, lr=1e-3)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    return {"case": "mlp", "steps": steps, "train_step_ms": ms,
            "train_step_tflops": 6.0 * 256 * net.param_count / (ms * 1e-3) / 1e12}


def main(argv=None) -> None:
    p = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    p.add_argument("case", choices=["fem", "gn", "mlp"])
    p.add_argument("--frames", type=int, default=4)
    p.add_argument("--reps", type=int, default=2)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--gn-factor", choices=["fp64", "fp32-refined"], default="fp64")
    a = p.parse_args(argv)
    if a.case == "fem":
        out = case_fem(a.frames, a.reps)
    elif a.case == "gn":
        out = case_gn(a.frames, a.gn_factor, a.reps)
    else:
        out = case_mlp(a.steps)
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
