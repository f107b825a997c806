"""The multi-GPU path of bench.py is replicas only (one image per rank, no
collective in the data path): its only cross-rank steps are the barrier and
the max over ranks of the timed region, checked here with world_size 2 on
the gloo backend (CPU)."""
import os
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 10.0 + 5.0 * rank  # rank 1 is the slow one
        dist.barrier()
        worst = bench.max_over_ranks(ms, "cpu")
        value = bench.replica_throughput(world, 4, 1_000_000_000, worst)
        q.put((rank, worst, value))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, worst, value in res:
        assert worst == pytest.approx(15.0)
        # 2 ranks x 4 steps x 1 GB in 15 ms
        assert value == pytest.approx(2 * 4 * 1.0 / 0.015)
