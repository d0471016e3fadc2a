"""The multi-rank path of the benchmark on CPU (world size 2, gloo): replicas
only -- every rank reconstructs its own seeded frames, and the whole-job
figures are the slowest rank's time and the frames of all ranks."""
import os
import socket

import numpy as np
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    total, done = bench.aggregate_over_ranks(10.0 * (rank + 1), 3 + rank, world, "cpu")
    q.put((rank, total, done, bench.rank_frame_seed(rank, 0)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_aggregation_and_disjoint_frames():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    results.sort()
    for rank, total, done, _ in results:
        assert total == 20.0 and done == 7.0, (rank, total, done)
    seeds = [r[3] for r in results]
    assert len(set(seeds)) == 2
    import sys
    sys.path.insert(0, ROOT)
    import bench
    cent = np.random.default_rng(0).uniform(-0.7, 0.7, (500, 2))
    f0 = bench.synthetic_frames(cent, 4, seeds[0])
    f1 = bench.synthetic_frames(cent, 4, seeds[1])
    assert not np.array_equal(f0, f1)


def test_single_rank_needs_no_process_group():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.aggregate_over_ranks(12.5, 4, 1, "cpu") == (12.5, 4.0)
