"""The multi-GPU path of bench.py on CPU: two gloo ranks.

Instances shard across ranks with no collective on the data path.  The only
cross-rank step is the max of the per-rank step time, and the reported rate
counts all ranks' instances against that max.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = 100.0 + 50.0 * rank          # rank 1 is the slow one
    m = bench.max_over_ranks(ms, dist)
    rate = bench.job_rate(64, 10, world, m)
    out.put((rank, m, rate))
    dist.destroy_process_group()


def test_two_gloo_ranks_max_time_and_rate():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29400 + (os.getpid() % 500)
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, m, rate in res:
        assert m == 150.0
        assert rate == pytest.approx(64 * 10 * 2 / 0.150)


def test_single_rank_is_local():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5, None) == 12.5
    assert bench.job_rate(8, 5, 1, 1000.0) == 40.0
