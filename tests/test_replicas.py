"""Multi-GPU is replicas only: every rank develops its own images and no data
crosses ranks. What the job reports across ranks is host logic, checked here
with two gloo ranks on the CPU: the slowest rank's time, the sum of the ranks'
work, and the whole-job rate bench.py reports (every rank's megapixels over
the slowest rank's time)."""
import os
import socket

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import sys
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world)})
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        seconds = 1.0 + rank            # rank 1 is the slower replica
        mpix = 100.0 * (rank + 1)       # and did more work
        q.put((rank, bench.over_ranks(seconds, "max"), bench.over_ranks(mpix, "sum"),
               bench.replica_rate(mpix, seconds)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replica_reductions_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, slowest, work, rate in res:
        assert slowest == 2.0 and work == 300.0
        assert rate == pytest.approx(150.0)   # 300 MP over the slowest rank's 2 s


def test_single_process_reductions_are_identities():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.over_ranks(3.5, "max") == 3.5 and bench.over_ranks(2.0, "sum") == 2.0
    assert bench.replica_rate(240.0, 2.0) == 120.0
