"""The multi-GPU path of bench.py on CPU: two gloo ranks.

Instances shard across ranks with no collective on the data path.  The only
cross-rank step is the max of the per-rank step time, and the reported rate
counts all ranks' instances against that max.  Each rank draws its own
instances (the workload seed plus its rank, as bench.py does) and evaluates
them alone: here with the CPU oracle standing in for the rank's plan, and the
gathered results must equal one process evaluating every shard.
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


N_SH, LV_SH, SEED_SH, B_SH = 6, 5.0, 41, 3


def _shard_Q(rank):
    """Q = conserve(ComputeQ(f, f)) of the instances of one rank's shard."""
    import numpy as np
    from oracle import pyoracle as po
    from spectralbte_gb300.workloads import two_maxwellian_batch
    g = po.Grid(N_SH, LV_SH, "0d")
    W = po.weights_iso(g, 1.0)
    cons = po.Conservation(g)
    f = two_maxwellian_batch(g.v, B_SH, SEED_SH + rank)
    return f, np.stack([cons(po.computeQ(g, W, f[b])) for b in range(B_SH)])


def _shard_rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    f, Q = _shard_Q(rank)
    got = [None] * world
    dist.all_gather_object(got, (rank, f, Q))
    out.put(got if rank == 0 else None)
    dist.destroy_process_group()


def test_two_gloo_ranks_evaluate_disjoint_shards():
    import numpy as np
    import torch.multiprocessing as mp
    sys.path.insert(0, ROOT)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29900 + (os.getpid() % 90)
    procs = [ctx.Process(target=_shard_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    gathered = next(r for r in res if r is not None)
    assert [r for r, _, _ in gathered] == [0, 1]
    assert not np.allclose(gathered[0][1], gathered[1][1])   # distinct instances
    for rank, f, Q in gathered:
        f1, Q1 = _shard_Q(rank)
        assert np.array_equal(f, f1)
        assert np.array_equal(Q, Q1)
