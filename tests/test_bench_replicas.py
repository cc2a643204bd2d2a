"""bench.py with N > 1: independent replicas, one per GPU, whose timed region ends in
a maximum over ranks (the replicas exchange nothing else).  Run here as two gloo
ranks on the CPU."""
import os
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dev, wall = bench.max_over_ranks(1.0 + rank, 10.0 - rank, dist)
        q.put((rank, dev, wall))
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_max_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = sorted(q.get(timeout=100) for _ in ps)
    for p in ps:
        p.join(timeout=30)
        assert p.exitcode == 0
    assert got == [(0, 2.0, 10.0), (1, 2.0, 10.0)]


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.0, 4.0, None) == (3.0, 4.0)
