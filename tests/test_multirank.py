"""Two-rank (gloo, CPU) tests of the multi-GPU path's host logic.

One search does not shard (every DVND iteration ends in a global greedy
merge), so N GPUs run independent replicas: each rank times its own steps,
the job's throughput is the sum of the work over the slowest rank's time, and
independent searches (batched and served forms) are partitioned by index
with no collective on the data path.  Here the ranks are CPU processes
joined by gloo, and the oracle stands in for the GPU work.
"""
import os
import socket
import sys

import numpy as np
import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import bench
    import oracle as orc

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        # Replica timing contract: per-rank work and times, sum and max over ranks.
        work = [10.0 * (rank + 1), 1.0]
        times = [0.5 + rank, 2.0 - rank]
        tot = bench.reduce_sum(work, world)
        tmax = bench.reduce_max(times, world)
        # Searches partitioned by index; results gathered for the check.
        jobs = []
        for j in bench.shard(7, world, rank):
            n = 20 + 3 * j
            x, y = orc.uniform_instance(n, 40 + j)
            t, st = orc.dvnd(orc.random_perm_tour(n, 40 + j), orc.dist(x, y, True))
            jobs.append((j, t.tolist(), st["cost"]))
        gathered = [None] * world
        dist.all_gather_object(gathered, jobs)
        q.put((rank, tot, tmax, gathered))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_and_shard():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    port = _free_port()
    q = mp.Queue()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {}
    for _ in range(2):
        rank, tot, tmax, gathered = q.get(timeout=120)
        out[rank] = (tot, tmax, gathered)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank in (0, 1):
        tot, tmax, gathered = out[rank]
        assert tot == [30.0, 2.0]          # 10 + 20 units of work, two steps
        assert tmax == [1.5, 2.0]          # the slowest rank's times
        by_job = {j: (t, c) for part in gathered for j, t, c in part}
        assert sorted(by_job) == list(range(7))  # every search exactly once
        assert all(len(part) in (3, 4) for part in gathered)
        for j in range(7):
            n = 20 + 3 * j
            x, y = oracle.uniform_instance(n, 40 + j)
            t, st = oracle.dvnd(oracle.random_perm_tour(n, 40 + j), oracle.dist(x, y, True))
            assert np.array_equal(np.array(by_job[j][0]), t) and by_job[j][1] == st["cost"]
