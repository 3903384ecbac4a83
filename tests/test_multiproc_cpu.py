"""The multi-GPU path of bench.py (replicas: one process per GPU, no
collective on the data path) with two gloo ranks on the CPU: ranks render
different cameras, the job time is the slowest rank's (max over ranks), and
the reported throughput counts every rank's rays."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r, _ = bench.dist_env()
        t = bench.max_over_ranks(0.5 + r)               # rank 1 is the slower one
        q.put((r, w, t, bench.job_throughput(640000, 10, w, t),
               [bench.frame_index(i, r) for i in range(3)]))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_rank_replicas_reduce_with_max_over_ranks():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out)
    assert all(o[2] == 1.5 for o in out)                  # both see the slowest rank's time
    assert all(o[3] == pytest.approx(640000 * 10 * 2 / 1.5) for o in out)
    assert set(out[0][4]).isdisjoint(out[1][4])           # the replicas render different frames


def test_single_process_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(0.25) == 0.25
    assert bench.job_throughput(100, 4, 1, 2.0) == 200.0
