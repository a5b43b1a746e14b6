"""Multi-rank host logic on CPU (gloo, world size 2): each rank runs its own
sequence (weak scaling, no data-path collective); the job's time is the max
over ranks and the throughput counts every rank's frames."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    # a CPU test on any machine: no device visible, so the ranks use gloo
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "CUDA_VISIBLE_DEVICES": ""})
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    import torch.distributed as dist
    r, w, _ = bench.dist_init()
    assert (r, w) == (rank, world) and dist.get_backend() == "gloo"
    local_ms = 100.0 + 50.0 * rank          # rank 1 is the slower one
    mx = bench.reduce_max(local_ms, w)
    bench.barrier(w)
    seed = 1000 + r                          # bench.run_ours: one sequence per rank
    q.put((r, mx, seed))
    dist.destroy_process_group()


def test_two_gloo_ranks_max_time_and_distinct_sequences():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert [m for _, m, _ in res] == [150.0, 150.0]       # both ranks see the max
    assert len({s for _, _, s in res}) == 2                # independent sequences
    steps, world = 10, 2
    value = world * steps / (150.0 / 1e3)                  # bench.py's whole-job frames/s
    assert abs(value - 133.333) < 1e-2
