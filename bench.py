#!/usr/bin/env python3
"""EIT reconstruction benchmark on GB300 (and the CPU reference arm).

Workload (one "step"): reconstruct a batch of conductivity frames on the
20k-node disk (80 rings: 19441 nodes, 38400 triangles), 32 electrodes with
adjacent drive / adjacent measurement (1024 voltages per frame), 2.5D model
with 8 axial harmonics (height 4, k_j = j*pi/2), logarithmic (dB)
conductivity, until every frame's relative data residual
||V_meas - V(sigma)|| / ||V_meas|| is at most 1e-3.  Synthetic, seeded data:
1-3 circular inclusions (radius U(0.05, 0.3), contrast log-uniform in
[0.1, 10]) on a 1 S/m background; V_meas from the forward model with FP64
refinement to 1e-9 (noise-free).

The headline value is the learned path.  Each frame's Gauss-Newton start is
the linear one-step GN prior from the homogeneous point plus a network's
correction.  The network is trained before the timed region on pairs the
forward solver generates, with targets where batched GN from the prior
converges.  Batched GN then iterates to the target; a frame whose start does
not lower the residual restarts from the homogeneous distribution.  The same
frames are also timed on the prior alone, on the plain batched GN path and
one frame at a time.  The metric is frames/s (frames that reach the target
per second).  The line also carries the CG SpMM bandwidth, the roofline of
the dominant kernel, the tensor-core J J^T rate and the CPU baseline.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

`--workload uneven` times the batch of uneven meshes instead: 64 ring meshes
with R ~ U{20..100} rings and 16 or 32 electrodes (seed 3), 4 harmonics
(height 4), 16 frames per mesh of a moving circular inclusion (radius
U(0.1, 0.3), contrast log-uniform in [0.1, 10]); one step = the forward
solves of all meshes and frames in the same CG launches.  Its line reports
mesh-frames/s, the CG bandwidth against the HBM roofline and the same solves
issued one mesh at a time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "EIT frames/s to 1e-3 rel residual: learned+batched vs plain GN; SpMV GB/s"
UNIT = "frames/s"


def parse_args():
    p = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    p.add_argument("--workload", choices=["gn", "uneven"], default="gn",
                   help="gn: learned/plain GN reconstruction (default); uneven: batch of uneven meshes")
    p.add_argument("--meshes", type=int, default=64, help="uneven workload: meshes per step")
    p.add_argument("--mesh-frames", type=int, default=16, help="uneven workload: frames per mesh")
    p.add_argument("--frames", type=int, default=32, help="frames per step per GPU")
    p.add_argument("--rings", type=int, default=80)
    p.add_argument("--electrodes", type=int, default=32)
    p.add_argument("--components", type=int, default=8)
    p.add_argument("--height", type=float, default=4.0)
    p.add_argument("--target", type=float, default=1e-3)
    p.add_argument("--lam-rel", type=float, default=2e-2,
                   help="Tikhonov lambda relative to the RMS row norm of J at the reference")
    p.add_argument("--max-gn", type=int, default=10)
    p.add_argument("--tol", type=float, default=1e-5, help="CG relative tolerance of the GN forward solves")
    p.add_argument("--preconditioner", choices=["jacobi", "two-level"], default="two-level",
                   help="CG preconditioner of every GPU solve (jacobi = the reference's)")
    p.add_argument("--gn-warm-start", choices=["homogeneous", "cold"], default="homogeneous",
                   help="initial fields of each GN solve's first forward solve (and of the training-pair solves)")
    p.add_argument("--gn-factor", choices=["fp32-refined", "fp64"], default="fp32-refined",
                   help="factor of J J^T + mu I in every Gauss-Newton update (mpf_solve_opts.gn_factor): the FP32 "
                        "factor with FP64 refinement (FP64 factor where it fails), or the FP64 factor")
    p.add_argument("--accept-tol", type=float, default=0.0,
                   help="CG tolerance of the learned start's acceptance solve in the timed steps "
                        "(mpf_solve_opts.accept_tol; 0: the full tolerance)")
    p.add_argument("--accept-study-tol", type=float, default=1e-4,
                   help="untimed study after the timed steps: the learned path again with this acceptance "
                        "tolerance, its decisions and step time against the timed run's (0: skip)")
    p.add_argument("--accept-margin", type=float, default=0.1)
    p.add_argument("--cpu-threads", type=int, default=0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cg-shapes", type=str, default="",
                   help="fix the CG launch shapes 'spmm,update,direction' (codes of mpf_eit_cg_variants) "
                        "instead of autotuning")
    p.add_argument("--train-pairs", type=int, default=16384,
                   help="training pairs of the learned warm start, generated by the forward solver")
    p.add_argument("--epochs", type=int, default=80)
    p.add_argument("--train-tol", type=float, default=1e-4,
                   help="CG tolerance of the training-pair and label solves (their inputs carry 60 dB noise)")
    p.add_argument("--save-network", type=str, default="", help="write the trained network to this checkpoint")
    p.add_argument("--load-network", type=str, default="",
                   help="start from this checkpoint (MLP.save) instead of training a network")
    p.add_argument("--hidden", type=int, default=2048, help="hidden width of the warm-start network")
    p.add_argument("--learned-prior", choices=["on", "off"], default="on",
                   help="on: the network learns the correction to the linear one-step GN prior "
                        "(mpf_eit_learned_prior); off: it predicts gamma alone")
    p.add_argument("--labels", choices=["gn", "truth"], default="gn",
                   help="training targets with the prior: gn = where batched GN from the prior converges "
                        "(learned.gn_labels), truth = the generating conductivity")
    p.add_argument("--single-frames", type=int, default=4,
                   help="frames per step timed one at a time on the plain GN path (0: skip)")
    p.add_argument("--profile-only", action="store_true",
                   help="only time the CG kernels (all groups active) on --frames frames; for ncu captures")
    return p.parse_args()


# ---------------------------------------------------------------------------
def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def synthetic_frames(centroids: np.ndarray, count: int, seed: int) -> np.ndarray:
    """Held-out log-conductivity frames in dB (v = 10 log10(sigma / 1 S/m)):
    the training pairs' family (1-3 disks, radius U(0.05, 0.3), contrast
    log-uniform in [0.1, 10], centres uniform over the disk that keeps them
    inside) from seeds the training never uses."""
    from mpflow_gb300.learned import inclusion_frames
    return inclusion_frames(centroids, count, np.random.default_rng(10_000_019 + seed))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def measured_bf16_tflops():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            return float(json.load(fh)["bf16_tflops"]), "measured"
    except (OSError, KeyError, ValueError):
        return 1900.0, "fallback"


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch and
# per (frame, harmonic) group of the three CG iteration kernels on the
# 80-ring, 32-electrode workload (32 right-hand sides per group), from one ncu
# capture of `python bench.py --profile-only --frames 16 --steps 3
# --cg-shapes 90,28,19` (112 groups; summary and full command in
# profiles/cg_kernels_R80_F16.md).  Traffic grows with the group count, so a
# launch of G groups moves G times these bytes.
CG_DRAM_BYTES_PER_GROUP = {"k_spmm_halo": 4.96e6, "k_update": 7.12e6, "k_direction": 12.00e6}


# ---------------------------------------------------------------------------
def build_problem(a):
    import mpflow_gb300 as mp
    mesh = mp.IrregularMesh.ring(a.rings)
    ports = mp.Ports.circularBoundary(a.electrodes, 0.1, mesh)
    pat = mp.adjacent_pattern(a.electrodes)
    src = mp.Sources(mp.OPEN, 1e-3, ports, pat, pat)
    return mesh, ports, pat, src


def reference_gn_frame(a, s, v_true):
    """One frame reconstructed by the oracle's Gauss-Newton loop (FP64): the
    forward model at the iterate, the data residual against the target, and
    the dual regularised update, from the homogeneous start.  Returns
    (seconds, updates, converged)."""
    import oracle
    Vm, _, _ = oracle.eit_forward(s, v_true, tol=1e-9, want_jacobian=False, exact=True)
    vm = oracle.flatten_measurement(Vm, s)
    t0 = time.perf_counter()
    v = np.zeros_like(v_true)
    n_up, lam, ok = 0, None, False
    for it in range(a.max_gn + 1):
        V, J, _ = oracle.eit_forward(s, v, tol=a.tol, exact=True)
        y = vm - oracle.flatten_measurement(V, s)
        ok = bool(np.linalg.norm(y) / np.linalg.norm(vm) <= a.target)
        if ok or it == a.max_gn:
            break
        if lam is None:
            lam = a.lam_rel * np.linalg.norm(J) / np.sqrt(J.shape[0])
        v = v + oracle.inverse_dual(J, y, 1.0, lam)
        n_up += 1
    return time.perf_counter() - t0, n_up, ok


def cpu_baseline(a, frame):
    """The oracle's Gauss-Newton loop on one frame of the timed workload, on
    all host cores: frames/s = 1 / seconds."""
    import oracle
    if a.cpu_threads > 0:
        oracle.set_threads(a.cpu_threads)
    s, _ = oracle_problem(a)
    dt, n_up, ok = reference_gn_frame(a, s, frame.astype(np.float64))
    return {"value": 1.0 / dt, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
            "sample": (f"1 frame (the first of the first timed step), FP64 Gauss-Newton from the homogeneous start "
                       f"to the target: {n_up} updates, {dt:.2f} s, converged {ok}")}


def oracle_problem(a):
    """The workload's mesh, ports and model built by the oracle alone (the
    FP64 restatement of the reference), so that the reference arm loads none
    of this library's compiled code."""
    import oracle
    nodes, elements = oracle.ring_mesh(a.rings)
    edges, _, boundary = oracle.mesh_edges(nodes, elements)
    ports = oracle.circular_ports(nodes, elements, edges, boundary, a.electrodes, 0.1)
    pat = oracle.adjacent_pattern(a.electrodes)
    s = oracle.Setup(nodes, elements, edges, boundary, ports, pat, pat, np.full(a.electrodes, 1e-3), ref=1.0,
                     logarithmic=True, components=a.components, height=a.height)
    return s, nodes[elements].mean(axis=1)


def run_reference(a):
    """--impl reference: the reference's numerics (the FP64 oracle, all host
    threads) on the same workload.  Each step reconstructs a bounded sample of
    the GPU arm's step: its first frame (the same seed), by the reference's
    Gauss-Newton loop (src/solver/solver.cpp:196-225 around
    src/models/eit.cpp:139-213 and the dual form of src/solver/inverse.cpp:
    60-238) from the homogeneous start to the same target."""
    rank, world, _ = dist_env()
    if world > 1 and rank != 0:
        return
    import oracle
    if a.cpu_threads > 0:
        oracle.set_threads(a.cpu_threads)
    s, cent = oracle_problem(a)
    times, iters, conv = [], [], 0
    for step in range(a.warmup + a.steps):
        v_true = synthetic_frames(cent, a.frames, seed=rank_frame_seed(0, step))[0].astype(np.float64)
        dt, n_up, ok = reference_gn_frame(a, s, v_true)
        if step >= a.warmup:
            times.append(dt)
            iters.append(n_up)
            conv += int(ok)
    value = conv / sum(times)
    sample = (f"1 frame per step (the first frame of the GPU arm's step, same seed), FP64 Gauss-Newton from the "
              f"homogeneous start to the target, {np.mean(iters):.2f} updates mean, {conv}/{len(times)} converged")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded inclusion frames, noise-free)",
        "config": workload_config(a, a.frames),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_config(a, frames):
    return {"workload": (f"EIT 2.5D GN reconstruction: ring mesh {a.rings} rings (19441 nodes, 38400 "
                         f"triangles at 80), {a.electrodes} electrodes adjacent/adjacent, "
                         f"{a.components} harmonics (height {a.height}), log-conductivity, 1-3 inclusions "
                         "r U(0.05,0.3) contrast log-U[0.1,10]"),
            "frames_per_step_per_gpu": frames, "target_rel_residual": a.target,
            "target_data": "noise-free held-out frames (60 dB noise only on the training pairs)",
            "lambda_rel": a.lam_rel, "cg_tol": a.tol, "jacobian": "exact 2.5D derivative",
            "gn_factor": a.gn_factor,
            "l2": "CG working set > L2 (129 MB) at >= 8 frames per step"}


def aggregate_over_ranks(total_ms, done, world, device):
    """Whole-job figures of a replicas-only run: the slowest rank's time and
    the frames all ranks finished (no collective on the data path; these two
    reductions only report)."""
    if world <= 1:
        return float(total_ms), float(done)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(total_ms)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    n = torch.tensor([float(done)], device=device, dtype=torch.float64)
    dist.all_reduce(n)
    return float(t.item()), float(n.item())


def rank_frame_seed(rank, step):
    """Seed of the held-out frames of one rank and step: every rank
    reconstructs its own frames."""
    return 1000 * (rank + 1) + step


def timed_steps(nsteps, warmup, fn, barrier, stream, torch, lib):
    """Run fn(step) for every step between barriers, CUDA events around each
    call on `stream`; returns (per-step ms of the timed steps, their results,
    kernel launches inside the timed steps)."""
    times, results, launches = [], [], 0
    for s in range(nsteps):
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = lib.mpf_kernel_launches()
        e0.record(stream)
        r = fn(s)
        e1.record(stream)
        barrier()
        if s >= warmup:
            times.append(e0.elapsed_time(e1))
            results.append(r)
            launches += lib.mpf_kernel_launches() - l0
    return times, results, launches


def run_gb300(a):
    import torch
    import torch.distributed as dist
    import mpflow_gb300 as mp
    from mpflow_gb300.learned import (generate_pairs, gn_labels, inclusion_frames, round_up, train_warm_start,
                                      zero_network)

    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group(backend="nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    mesh, ports, pat, src = build_problem(a)
    E = mesh.elements.shape[0]
    cent = mesh.nodes[mesh.elements].mean(axis=1)
    model = mp.EIT(mesh, src, 1.0, components=a.components, height=a.height, logarithmic=True,
                   device=local, exact_jacobian=True)
    F = a.frames
    nsteps = a.warmup + a.steps
    if a.cg_shapes:
        model.cg_variants(F, set=[int(x) for x in a.cg_shapes.split(",")])
    if a.profile_only:
        v = torch.tensor(synthetic_frames(cent, F, seed=7), device=dev)
        ms, by = model.profile_cg(v, reps=max(a.steps, 1))
        names = ["k_spmm_halo" if model.cg_variants(F)[0] >= 72 else "k_spmm_dot", "k_update", "k_direction"]
        print(json.dumps({"profile_only": True, "frames": F, "groups": F * model.info["active_components"],
                          "cg_shapes": model.cg_variants(F).tolist(),
                          "ms": dict(zip(names, ms.tolist())),
                          "gbs": dict(zip(names, (by / ms / 1e6).tolist())),
                          "algorithmic_bytes": dict(zip(names, by.tolist())),
                          "cg_loop_overhead": model.profile_cg_loop(v, graphs=8)}), flush=True)
        return
    lib = mp.lib()
    # held-out frames and their noise-free measurements (untimed)
    truth = [synthetic_frames(cent, F, seed=rank_frame_seed(rank, s)) for s in range(nsteps)]
    ref_opts = mp.SolveOptions(tol=1e-5, refine_tol=1e-9, max_iter=6000, preconditioner=a.preconditioner)
    vmeas = [model.solve(torch.tensor(truth[s], device=dev), ref_opts).contiguous() for s in range(nsteps)]
    opts = mp.SolveOptions(tol=a.tol, max_iter=6000, preconditioner=a.preconditioner)
    _, J0 = model.solve(torch.zeros((1, E), device=dev), opts, jacobian=True)
    # GN paths: the first forward solve of every frame starts from the fields of
    # the homogeneous distribution (solved once per model)
    gn_opts = mp.SolveOptions(tol=a.tol, max_iter=6000, preconditioner=a.preconditioner,
                              warm_start="homogeneous" if a.gn_warm_start == "homogeneous" else 0,
                              gn_factor=a.gn_factor)
    # the learned path: acceptance solve at accept_tol (the plain and
    # prior-only paths have no acceptance solve; for them it changes nothing)
    learned_opts = mp.SolveOptions(tol=a.tol, max_iter=6000, preconditioner=a.preconditioner,
                                   warm_start="homogeneous" if a.gn_warm_start == "homogeneous" else 0,
                                   gn_factor=a.gn_factor, accept_tol=a.accept_tol, accept_margin=a.accept_margin)
    lam = a.lam_rel * float(J0.norm() / np.sqrt(J0.shape[1]))
    del J0

    # learned warm start: pairs from the forward solver, training on the GPU (untimed, reported)
    train_opts = mp.SolveOptions(tol=a.train_tol, max_iter=6000, preconditioner=a.preconditioner,
                                 warm_start="homogeneous" if a.gn_warm_start == "homogeneous" else 0,
                                 gn_factor=a.gn_factor)
    if a.load_network:
        a.train_pairs = 0
    t0 = time.perf_counter()
    gtrain = inclusion_frames(cent, max(a.train_pairs, 64), np.random.default_rng(5 + 7919 * rank))
    Vtr, gtr = generate_pairs(model, gtrain, batch=128, options=train_opts)
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t0
    L = Vtr.shape[1] * Vtr.shape[2]
    use_prior = a.learned_prior == "on"
    prior_s = None
    if use_prior:
        t0 = time.perf_counter()
        model.learned_prior(lam)
        prior_s = time.perf_counter() - t0
    label_s, label_conv = None, None
    if use_prior and a.labels == "gn" and not a.load_network:
        t0 = time.perf_counter()
        gtr, label_conv = gn_labels(model, Vtr, lam, target=a.target, max_iters=4, batch=128, options=train_opts)
        torch.cuda.synchronize()
        label_s = time.perf_counter() - t0
    if a.load_network:
        net = mp.MLP.load(a.load_network, device=local)
        losses, train_s = [float("nan")], float("nan")
    else:
        net = mp.MLP(L, a.hidden, a.hidden, round_up(E, 128), seed=17 + rank)
        losses, train_s = train_warm_start(model, net, Vtr, gtr, epochs=a.epochs, batch=256, lr=1e-3,
                                           snr_db=60.0, seed=rank, prior=use_prior)
    if a.save_network and rank == 0:
        net.save(a.save_network)
    net0 = zero_network(L, round_up(E, 128)) if use_prior else None
    train_steps = a.epochs * max(1, a.train_pairs // 256) if not a.load_network else 0
    # the training step alone (mpf_mlp_train_step, CUDA events; a throwaway
    # network of the same shape on the same pairs): what the kernels sustain
    # without the per-epoch work (noise, network inputs, prior targets)
    probe = mp.MLP(L, a.hidden, a.hidden, round_up(E, 128), seed=99, device=local)
    Xp = model.learned_input(Vtr)
    batches = [torch.randint(0, Vtr.shape[0], (256,), device=dev, dtype=torch.int32) for _ in range(23)]
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    for k, rows in enumerate(batches):
        if k == 3:  # three untimed steps first
            ev[0].record(torch.cuda.current_stream())
        probe.train_step(Xp, gtr, rows=rows, valid=E, lr=1e-4)
    ev[1].record(torch.cuda.current_stream())
    torch.cuda.synchronize()
    train_step_ms = ev[0].elapsed_time(ev[1]) / (len(batches) - 3)
    del probe, Xp, batches
    del Vtr, gtr

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    stream = torch.cuda.current_stream()

    def learned_step(s):
        _, it, res, acc, st = model.gn_solve_learned(net, vmeas[s], lam, target=a.target, max_iters=a.max_gn,
                                                     options=learned_opts)
        return it, acc, st

    def prior_step(s):
        _, it, res, acc, st = model.gn_solve_learned(net0, vmeas[s], lam, target=a.target, max_iters=a.max_gn,
                                                     options=gn_opts)
        return it, acc, st

    def plain_step(s):
        g = torch.zeros((F, E), device=dev)
        it, res, st = model.gn_solve(g, vmeas[s], lam, target=a.target, max_iters=a.max_gn, options=gn_opts)
        return it, None, st

    def single_step(s):
        its, conv = [], 0
        for f in range(a.single_frames):
            g = torch.zeros((1, E), device=dev)
            it, res, st = model.gn_solve(g, vmeas[s][f:f + 1], lam, target=a.target, max_iters=a.max_gn,
                                         options=gn_opts)
            its.append(int(it[0]))
            conv += int(st.frames_converged)
        return np.array(its), None, conv

    def summarise(times, results, frames_per_step):
        done = float(sum(int(r[2].frames_converged) if hasattr(r[2], "frames_converged") else int(r[2])
                         for r in results))
        total_ms, done = aggregate_over_ranks(float(np.sum(times)), done, world, dev)
        its = np.concatenate([r[0] for r in results])
        sts = [r[2] for r in results if hasattr(r[2], "solves_fp32")]
        solves = ({"fp32_refined": sum(t.solves_fp32 for t in sts) / len(sts),
                   "fp64": sum(t.solves_fp64 for t in sts) / len(sts)} if sts else None)
        return {"value": done / (total_ms / 1e3), "ms_per_step": float(np.mean(times)),
                "gn_solves_per_step": solves,
                "gn_updates_mean": float(its.mean()), "no_update_fraction": float(np.mean(its == 0)),
                "frames_converged_fraction": done / (frames_per_step * world * len(results))}

    def with_phases(fn):
        # the phase timer restarts at the first timed step and runs through the rest
        def run(s):
            if s == a.warmup:
                model.phase_times(True)
            return fn(s)
        return run

    with ClockSampler(local) as clocks:
        t_l, r_l, launches = timed_steps(nsteps, a.warmup, with_phases(learned_step), barrier, stream, torch, lib)
        phases_l, _ = model.phase_times(False)
        t_p, r_p, _ = timed_steps(nsteps, a.warmup, with_phases(plain_step), barrier, stream, torch, lib)
        phases_p, _ = model.phase_times(False)
        prior_only = None
        if use_prior:
            t_q, r_q, _ = timed_steps(nsteps, a.warmup, prior_step, barrier, stream, torch, lib)
            prior_only = summarise(t_q, r_q, F)
        single = None
        if a.single_frames > 0:
            t_s, r_s, _ = timed_steps(nsteps, a.warmup, single_step, barrier, stream, torch, lib)
            single = summarise(t_s, r_s, a.single_frames)
    learned = summarise(t_l, r_l, F)
    plain = summarise(t_p, r_p, F)
    accepted = float(np.mean(np.concatenate([r[1] for r in r_l])))

    # the looser acceptance solve against the timed run's decisions on the same
    # held-out frames (untimed by the step clock; CUDA events per call): the
    # accepted flags and updates per frame, CG iterations and step time
    accept_check = None
    study_tol = a.accept_study_tol if a.accept_study_tol > a.tol else 0.0
    if study_tol > 0.0 and study_tol != learned_opts.accept_tol:
        study_opts = mp.SolveOptions(tol=a.tol, max_iter=6000, preconditioner=a.preconditioner,
                                     warm_start="homogeneous" if a.gn_warm_start == "homogeneous" else 0,
                                     gn_factor=a.gn_factor, accept_tol=study_tol, accept_margin=a.accept_margin)
        same_acc = same_its = n_fr = 0
        cg_study = cg_timed = study_decided = 0
        study_ms = []
        for i, s in enumerate(range(a.warmup, nsteps)):
            barrier()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            _, it_s, _, acc_s, st_s = model.gn_solve_learned(net, vmeas[s], lam, target=a.target,
                                                             max_iters=a.max_gn, options=study_opts)
            e1.record(stream)
            barrier()
            study_ms.append(e0.elapsed_time(e1))
            it_t, acc_t, st_t = r_l[i]
            same_acc += int(np.sum(np.asarray(acc_t) == acc_s))
            same_its += int(np.sum(np.asarray(it_t) == it_s))
            n_fr += F
            cg_study += int(st_s.cg_iterations)
            cg_timed += int(st_t.cg_iterations)
            study_decided += int(st_s.accepted_loose)
        k = max(1, nsteps - a.warmup)
        accept_check = {"timed_accept_tol": learned_opts.accept_tol, "study_accept_tol": study_tol,
                        "accept_margin": a.accept_margin, "cg_tol": a.tol, "frames": n_fr,
                        "accepted_equal_fraction": same_acc / n_fr, "updates_equal_fraction": same_its / n_fr,
                        "study_decided_on_loose_fraction": study_decided / n_fr,
                        "cg_iterations_per_step": {"timed": cg_timed / k, "study": cg_study / k},
                        "ms_per_step": {"timed": float(np.mean(t_l)), "study": float(np.mean(study_ms))}}

    # end to end through the public API: host V_meas in, host sigma out (learned path)
    host_v = [v.cpu().pin_memory() for v in vmeas]
    host_out = torch.empty((F, E), dtype=torch.float32).pin_memory()
    e2e_ms, e2e_frames = [], 0
    for s in range(nsteps):
        barrier()
        t0 = time.perf_counter()
        vm = host_v[s].to(dev, non_blocking=True)
        g, _, _, _, st = model.gn_solve_learned(net, vm, lam, target=a.target, max_iters=a.max_gn,
                                                options=learned_opts)
        host_out.copy_(g, non_blocking=True)
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) * 1e3
        if s >= a.warmup:
            e2e_ms.append(dt)
            e2e_frames += int(st.frames_converged)
    e2e_total, e2e_done = aggregate_over_ranks(sum(e2e_ms), e2e_frames, world, dev)
    e2e_value = e2e_done / (e2e_total / 1e3)

    # device time per phase of one timed step (the library's CUDA-event phase
    # timer, mpf_eit_phase_times); the phases of a step add up to its time
    def breakdown(phases, times):
        per = {k: v / len(times) for k, v in phases.items()}
        total = sum(per.values())
        return {"ms_per_step": per, "sum_ms": total, "step_ms": float(np.mean(times)),
                "share": {k: v / total for k, v in per.items()} if total > 0 else None}

    phase_learned = breakdown(phases_l, t_l)
    phase_plain = breakdown(phases_p, t_p)

    # roofline of the CG iteration (the largest phase of the step): its three
    # kernels timed with CUDA events on the launching stream, every group active
    ms, by = model.profile_cg(torch.tensor(truth[0], device=dev), reps=10)
    gbs = by / ms / 1e6
    names = ["k_spmm_halo" if model.cg_variants(F)[0] >= 72 else "k_spmm_dot", "k_update", "k_direction"]
    peak, peak_kind = measured_peaks()
    groups = F * model.info["active_components"]
    traffic = [CG_DRAM_BYTES_PER_GROUP.get(n) for n in names]
    roofline = {"kernel": "CG iteration: " + " + ".join(names), "bound": "hbm",
                "achieved": float(by.sum() / ms.sum() / 1e6), "peak": peak, "unit": "GB/s",
                "frac": float(by.sum() / ms.sum() / 1e6 / peak), "peak_source": f"{peak_kind} hbm_gbs",
                "traffic": float(sum(traffic) * groups) if all(t is not None for t in traffic) else None,
                "algorithmic_bytes": float(by.sum()), "launch_ms": float(ms.sum()),
                "why": "the Krylov iterations are the largest phase of the timed step (phase_breakdown)"}
    cg_kernels = {n: {"ms": float(ms[i]), "algorithmic_bytes": float(by[i]), "gbs": float(gbs[i]),
                      "frac_of_hbm": float(gbs[i] / peak),
                      "dram_bytes": (traffic[i] * groups if traffic[i] is not None else None)}
                  for i, n in enumerate(names)}

    # launch and graph overhead of the CG loop: per-iteration time of the loop
    # as a solve runs it (graphs of 16 iterations, host convergence check
    # between graphs) against the same kernels timed one launch at a time
    cg_loop = model.profile_cg_loop(torch.tensor(truth[0], device=dev), graphs=8)

    # assembly and Jacobian kernels (HBM-bound), CUDA events on the launching stream
    fem_ms, fem_by = model.profile_fem(torch.tensor(truth[0], device=dev), reps=5)
    fem = {}
    for i, name in enumerate(["k_assemble", "k_jacobian"]):
        gbs_i = float(fem_by[i] / fem_ms[i] / 1e6)
        fem[name] = {"ms": float(fem_ms[i]), "algorithmic_bytes": float(fem_by[i]), "gbs": gbs_i,
                     "frac_of_hbm": gbs_i / peak, "frames": F}

    # J J^T of the GN step on the tensor cores at this workload's size (all
    # frames of a step in one launch), CUDA events
    rows_j = model.jacobian_rows
    jjt_ms = mp.profile_gram(F, rows_j, round_up(E, 64), reps=5)
    bf16_peak, bf16_kind = measured_bf16_tflops()
    jjt_tflops = 2.0 * rows_j * rows_j * E * F / (jjt_ms * 1e-3) / 1e12  # GEMM-equivalent flops
    nt = rows_j // 128  # 128 x 128 output tiles; only those on and above the diagonal are computed
    executed = jjt_tflops * 3.0 * (nt * (nt + 1) / 2) / (nt * nt)
    jjt = {"frames": F, "rows": rows_j, "elements": E, "ms": jjt_ms, "tflops_gemm_equivalent": jjt_tflops,
           "frac_of_bf16_peak_over_3": jjt_tflops / (bf16_peak / 3.0),
           "tflops_executed": executed, "frac_executed_of_bf16_peak": executed / bf16_peak,
           "peak_source": f"{bf16_kind} bf16_tflops (burst); 3 products hi.hi + hi.lo + lo.hi",
           "note": "upper-triangle tiles only, so the GEMM-equivalent rate can exceed peak / 3"}

    if rank != 0:
        return
    cpu = None
    if not a.no_cpu_baseline:
        cpu = cpu_baseline(a, truth[a.warmup][0])
    mlp_flops = 6.0 * 256 * net.param_count * train_steps
    line = {
        "metric": METRIC, "value": learned["value"], "unit": UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": learned["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (FP64 inner products and refinement, FP32 Cholesky refined in FP64, split-BF16 J J^T, "
                                      "BF16 network)",
        "data": "synthetic (seeded inclusion frames; V_meas noise-free from the FP64-refined forward model; "
                "training pairs from the forward model with 60 dB noise)",
        "config": workload_config(a, F),
        "method": ("learned warm start = linear one-step GN prior from the homogeneous point + trained network "
                   "correction" if use_prior else "learned warm start (network alone)")
                  + "; batched GN from it (plain GN restart per frame when the start does not lower the residual)",
        "cg_preconditioner": a.preconditioner,
        "gn_factor": a.gn_factor,
        "gn_first_solve_start": a.gn_warm_start,
        "gn_updates_mean": learned["gn_updates_mean"],
        "frames_converged_fraction": learned["frames_converged_fraction"],
        "accept_check": accept_check,
        "learned": {"accepted_fraction": accepted,
                    "gn_updates_saved_per_frame": plain["gn_updates_mean"] - learned["gn_updates_mean"],
                    "train_pairs": a.train_pairs, "pair_generation_s": gen_s, "epochs": a.epochs,
                    "train_s": train_s, "train_steps": train_steps, "loss_first": losses[0],
                    "loss_last": losses[-1], "network": f"{L}-{a.hidden}-{a.hidden}-{round_up(E, 128)} GELU",
                    "train_tflops": (mlp_flops / train_s / 1e12) if train_steps else None,
                    "train_step_ms": train_step_ms,
                    "train_step_tflops": 6.0 * 256 * net.param_count / (train_step_ms * 1e-3) / 1e12,
                    "train_tflops_what": "train_tflops: 6 x 256 x parameters x steps over the whole training "
                                         "loop (per-epoch noise, inputs and prior targets included); "
                                         "train_step_tflops: one mpf_mlp_train_step alone, CUDA events",
                    "train_cg_tol": a.train_tol, "loaded_network": a.load_network or None,
                    "labels": (("GN from the prior to the target (<= 4 updates; the prior where it does not "
                                "converge)") if label_s is not None else "generating conductivity"),
                    "label_s": label_s, "label_converged_fraction": label_conv,
                    "prior": ({"lambda": lam, "setup_s": prior_s,
                               "what": "J0^T (J0 J0^T + mu I)^-1 at the homogeneous point, FP64 Gram/Cholesky, "
                                       "applied as a split-BF16 tensor-core product (hi.hi + lo.hi + hi.lo)"} if use_prior else None),
                    "no_update_fraction": learned["no_update_fraction"]},
        "prior_only_gn_batched": prior_only,
        "plain_gn_batched": plain,
        "plain_gn_single_frame": single,
        "learned_vs_plain_batched": learned["value"] / plain["value"],
        "learned_vs_plain_single_frame": (learned["value"] / single["value"]) if single else None,
        "spmv_gbs": float(gbs[0]),
        "spmv": {"kernel": names[0], "gbs": float(gbs[0]), "frac_of_hbm": float(gbs[0] / peak), "target_frac": 0.70},
        "cg_kernels": cg_kernels,
        "cg_loop_overhead": cg_loop,
        "phase_breakdown": {"learned": phase_learned, "plain_gn_batched": phase_plain},
        "roofline": roofline,
        "jjt_tensor_core": jjt,
        "fem_kernels": fem,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": int(vmeas[0].numel() * 4), "d2h_bytes_per_step": int(F * E * 4)},
        "clocks": clocks.summary(),
        "gpu_launches": int(launches),
        "cg_variants": model.cg_variants(F).tolist(),
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


# ---------------------------------------------------------------------------
UNEVEN_METRIC = "EIT forward solves of 64 uneven meshes x 16 frames in one batch: mesh-frames/s; CG GB/s"
UNEVEN_UNIT = "mesh-frames/s"


def uneven_setup(a):
    """Seeded mesh sizes, electrode counts and moving-inclusion frames."""
    import mpflow_gb300 as mp
    rng = np.random.default_rng(3)
    rings = rng.integers(20, 101, size=a.meshes)
    elec = rng.choice([16, 32], size=a.meshes)
    meshes, frames = [], []
    for i in range(a.meshes):
        mesh = mp.IrregularMesh.ring(int(rings[i]))
        ports = mp.Ports.circularBoundary(int(elec[i]), 0.1, mesh)
        pat = mp.adjacent_pattern(int(elec[i]))
        src = mp.Sources(mp.OPEN, 1e-3, ports, pat, pat)
        cent = mesh.nodes[mesh.elements].mean(axis=1)
        r = rng.uniform(0.1, 0.3)
        contrast = np.exp(rng.uniform(np.log(0.1), np.log(10.0)))
        orbit = rng.uniform(0.0, 0.9 - r)
        phase = rng.uniform(0.0, 2 * np.pi)
        g = np.ones((a.mesh_frames, cent.shape[0]), np.float32)
        for f in range(a.mesh_frames):
            th = phase + 2 * np.pi * f / a.mesh_frames
            c = orbit * np.array([np.cos(th), np.sin(th)])
            g[f, np.linalg.norm(cent - c, axis=1) < r] = contrast
        meshes.append((mesh, ports, pat, src))
        frames.append(g)
    return rings, elec, meshes, frames


def uneven_config(a, rings, elec):
    return {"workload": (f"{a.meshes} ring meshes, rings U{{20..100}} and 16/32 electrodes (seed 3), "
                         f"adjacent/adjacent, 4 harmonics (height 4), {a.mesh_frames} frames per mesh: moving "
                         "inclusion r U(0.1,0.3), contrast log-U[0.1,10], linear conductivity"),
            "nodes_total": int(sum(1 + 3 * r * (r + 1) for r in rings)),
            "meshes_16_electrodes": int((elec == 16).sum()), "meshes_32_electrodes": int((elec == 32).sum()),
            "frames_per_mesh": a.mesh_frames, "cg_tol": a.tol, "preconditioner": a.preconditioner,
            "l2": "CG working set (GBs) far above L2 (129 MB)"}


def run_uneven(a):
    import torch
    import mpflow_gb300 as mp
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend="nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    rings, elec, meshes, frames = uneven_setup(a)
    models = [mp.EIT(m, src, 1.0, components=4, height=4.0, device=local) for m, _, _, src in meshes]
    batch = mp.EITBatch(models)
    gam = [torch.tensor(g, device=dev) for g in frames]
    opts = mp.SolveOptions(tol=a.tol, preconditioner=a.preconditioner)
    lib = mp.lib()
    stream = torch.cuda.current_stream()
    nsteps = a.warmup + a.steps

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    cg = []

    def batch_step(s):
        V = batch.solve(gam, opts)
        cg.append(batch.cg_stats())
        return V

    def sequential_step(s):
        return [m.solve(g, opts) for m, g in zip(models, gam)]

    mf = a.meshes * a.mesh_frames
    with ClockSampler(local) as clocks:
        t_b, _, launches = timed_steps(nsteps, a.warmup, batch_step, barrier, stream, torch, lib)
        t_s, _, _ = timed_steps(min(nsteps, a.warmup + 2), a.warmup, sequential_step, barrier, stream, torch, lib)
    iters = batch.iterations(a.mesh_frames)
    cg_ms = float(np.mean([c[0] for c in cg[a.warmup:]]))
    cg_bytes = float(np.mean([c[1] for c in cg[a.warmup:]]))

    def max_over_ranks(ms):
        return aggregate_over_ranks(ms, 0.0, world, dev)[0]

    total_b = max_over_ranks(float(np.sum(t_b)))
    total_s = max_over_ranks(float(np.sum(t_s)))
    value = mf * world * len(t_b) / (total_b / 1e3)
    seq_value = mf * world * len(t_s) / (total_s / 1e3)

    # end to end through the public API: pinned host frames in, host voltages out
    host_g = [g.cpu().pin_memory() for g in gam]
    e2e_ms = []
    h2d = sum(g.numel() * 4 for g in gam)
    d2h = 0
    for s in range(nsteps):
        barrier()
        t0 = time.perf_counter()
        gd = [h.to(dev, non_blocking=True) for h in host_g]
        V = batch.solve(gd, opts)
        Vh = [v.cpu() for v in V]
        torch.cuda.synchronize()
        if s >= a.warmup:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
        d2h = sum(v.numel() * 4 for v in Vh)
    e2e_value = mf * world * len(e2e_ms) / (max_over_ranks(float(np.sum(e2e_ms))) / 1e3)
    if rank != 0:
        return
    peak, peak_kind = measured_peaks()
    gbs = cg_bytes / cg_ms / 1e6
    cpu = None
    if not a.no_cpu_baseline:
        import oracle
        if a.cpu_threads > 0:
            oracle.set_threads(a.cpu_threads)
        i = int(np.argsort(rings)[len(rings) // 2])  # the median mesh, one frame
        mesh, ports, pat, _ = meshes[i]
        so = oracle.Setup(mesh.nodes, mesh.elements, mesh.edges, mesh.boundary, ports.edges, pat, pat,
                          np.full(int(elec[i]), 1e-3), ref=1.0, components=4, height=4.0)
        t0 = time.perf_counter()
        oracle.eit_forward(so, frames[i][0].astype(np.float64), tol=a.tol, want_jacobian=False)
        dt = time.perf_counter() - t0
        cpu = {"value": 1.0 / dt, "unit": UNEVEN_UNIT, "cores": oracle.num_threads(), "kind": "port",
               "sample": f"1 frame of the median mesh ({int(rings[i])} rings, {int(elec[i])} electrodes), FP64 "
                         f"Jacobi-PCG forward solve, {dt:.2f} s"}
    line = {
        "metric": UNEVEN_METRIC, "value": value, "unit": UNEVEN_UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": float(np.mean(t_b)), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (FP64 inner products)",
        "data": "synthetic (seeded meshes and moving-inclusion frames)",
        "config": uneven_config(a, rings, elec),
        "cg": {"ms": cg_ms, "algorithmic_bytes": cg_bytes, "gbs": gbs,
               "iterations_max": int(iters.max()), "iterations_mean": float(iters.mean()),
               "launch_shapes": batch.cg_variants(a.mesh_frames).tolist()},
        "roofline": {"kernel": "batched CG (k_spmm_dot + k_update + k_direction)", "bound": "hbm",
                     "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                     "peak_source": f"{peak_kind} hbm_gbs", "traffic": None},
        "one_mesh_at_a_time": {"value": seq_value, "ms_per_step": float(np.mean(t_s))},
        "batch_vs_one_mesh_at_a_time": value / seq_value,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": UNEVEN_UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "clocks": clocks.summary(),
        "gpu_launches": int(launches),
    }
    print(json.dumps(line), flush=True)


def main():
    a = parse_args()
    if a.impl == "reference":
        run_reference(a)
    elif a.workload == "uneven":
        run_uneven(a)
    else:
        run_gb300(a)


if __name__ == "__main__":
    main()
