"""The multi-rank bench path on CPU: two gloo ranks, each with its own
molecule shard (no data-path collective), max-over-ranks timing and the
whole-job aggregate.  Mirrors what torchrun + NCCL does on GPUs."""
import multiprocessing as mp
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    r, w, local, dist = bench.dist_setup()
    mols = bench.workload(r, 3)
    first_xyz = float(mols[0].xyz[0, 0])
    fake_ms = 10.0 * (r + 1)                 # the slower rank sets the job's time
    mx = bench.max_over_ranks(fake_ms, dist)
    value = bench.aggregate_throughput(w, 3, mx)
    bench.barrier_sync(dist)
    dist.destroy_process_group()
    q.put((r, w, first_xyz, mx, value))


@pytest.mark.timeout(120)
def test_two_gloo_ranks_shard_and_reduce():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=100) for _ in range(2))
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    (r0, w0, x0, m0, v0), (r1, w1, x1, m1, v1) = out
    assert (r0, r1) == (0, 1) and w0 == w1 == 2
    assert x0 != x1                          # each rank solves its own replicas
    assert m0 == m1 == 20.0                  # max over ranks
    assert v0 == v1 == pytest.approx(2 * 3 / 0.020)


def _shard_rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    from molds_gb300 import sharding
    from molds_gb300 import workloads as W
    r, w, local, dist = bench.dist_setup()
    # the uneven workload's basis sizes (random alkanes, N = 6 n + 2)
    n_all = np.array([6 * W.alkane_carbons(3_000_000 + j) + 2 for j in range(200)])
    shards = sharding.shard_by_cost(sharding.predicted_cost(n_all), w)
    everyone = [None] * w
    dist.all_gather_object(everyone, shards)
    dist.destroy_process_group()
    q.put((r, shards, everyone, n_all.tolist()))


@pytest.mark.timeout(120)
def test_two_gloo_ranks_split_uneven_batch_by_cost():
    """Each rank computes the same N^3-cost assignment of an uneven alkane
    batch without a data-path collective (checked here by gathering it); the
    shards are disjoint, cover the batch and are balanced far better than an
    equal-count split."""
    from molds_gb300 import sharding
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=100) for _ in range(2))
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    (_, s0, all0, n_all), (_, s1, all1, _) = out
    assert s0 == s1 == all0[0] == all1[1]
    flat = sorted(s0[0] + s0[1])
    assert flat == list(range(len(n_all)))
    cost = sharding.predicted_cost(n_all)
    loads = sharding.shard_loads(cost, s0)
    assert loads.max() <= cost.sum() / 2 * 1.01
    naive = sharding.shard_loads(cost, [list(range(0, len(n_all), 2)), list(range(1, len(n_all), 2))])
    assert loads.max() <= naive.max()
