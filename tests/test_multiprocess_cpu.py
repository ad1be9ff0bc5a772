"""The multi-rank host logic of bench.py on CPU: world size 2 over gloo (127.0.0.1).  A
single universe runs as independent replicas; a batch of universes shards by universe with
no collective on the data path; only the timing reduction (max over ranks) and the job's
interaction total (sum) cross ranks."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, counts, q):
    import torch.distributed as dist
    import bench
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = bench.shard_universes(counts, world, rank)
        local_ms = 10.0 + rank                    # stand-in timings: rank 1 is slower
        job_ms = bench.reduce_max(local_ms, dist)
        job_inter = bench.reduce_sum(int(np.asarray(counts)[mine].sum()), dist)
        q.put((rank, mine.tolist(), job_ms, job_inter))
    finally:
        dist.destroy_process_group()


def test_two_ranks_shard_universes_and_reduce_over_gloo():
    import torch.multiprocessing as mp
    counts = np.array([1024, 33, 5000, 1, 65536, 2048, 700, 4096, 12000, 9], np.int64)
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, counts, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    shards = [set(r[1]) for r in res]
    assert shards[0].isdisjoint(shards[1]) and shards[0] | shards[1] == set(range(counts.size))
    for r in res:
        assert r[2] == 11.0                        # max over ranks
        assert r[3] == counts.sum()                # every body counted once
    # balance: the heavier shard carries at most the largest universe more than the other
    cost = counts * np.log2(np.maximum(counts, 2))
    loads = [cost[list(s)].sum() for s in shards]
    assert abs(loads[0] - loads[1]) <= cost.max()


def _ensemble(counts, seed=5):
    from nbh import universe as U
    parts = [U.PlummerUniverseGenerator(seed=seed * 1000 + u).arrays(int(c)) for u, c in enumerate(counts)]
    return tuple(np.concatenate([p[k] for p in parts]) for k in range(7))


def _step_shard(arrs, counts, steps):
    """What one rank does with its shard, on the oracle: every universe of the shard loaded
    and stepped on its own (bench._oracles, the per-rank CPU path); the final state of each
    universe and the shard's interactions of the last step."""
    import argparse

    import bench
    args = argparse.Namespace(theta=0.5, eps=0.05, dt=0.01, vote_width=64)
    orc = bench._oracles(arrs, counts, args)
    for o in orc:
        assert o.step(steps) == 0
    return [o.state() for o in orc], sum(o.interactions for o in orc)


def _rank_step_main(rank, world, port, counts, steps, q):
    import torch.distributed as dist
    import bench
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = bench.shard_universes(counts, world, rank)
        arrs, sub = bench.select_universes(_ensemble(counts), counts, mine)
        states, inter = _step_shard(arrs, sub, steps)
        job_inter = bench.reduce_sum(inter, dist)
        q.put((rank, mine.tolist(), states, job_inter))
    finally:
        dist.destroy_process_group()


def test_two_ranks_step_their_shards_like_one_process():
    """Each of two gloo ranks selects its shard of an uneven ensemble and steps it (the
    oracle stands in for the GPU on CPU); the union of the ranks' universes equals one
    process stepping the whole batch, universe by universe and bit for bit, and the job's
    interaction total is the single-process total."""
    import torch.multiprocessing as mp
    counts = np.array([300, 33, 1500, 1, 700, 64, 65, 2000, 129, 900], np.int64)
    steps, world = 2, 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_step_main, args=(r, world, port, counts, steps, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=300) for _ in range(world)), key=lambda r: r[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    whole, total = _step_shard(_ensemble(counts), counts, steps)
    seen = set()
    for rank, mine, states, job_inter in res:
        assert job_inter == total
        for u, st in zip(mine, states):
            seen.add(u)
            for k in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az"):
                np.testing.assert_array_equal(st[k], whole[u][k], err_msg="universe %d %s" % (u, k))
    assert seen == set(range(counts.size))


def test_single_process_reductions_are_identity():
    import bench
    assert bench.reduce_max(3.5) == 3.5 and bench.reduce_sum(7) == 7
    counts = [5, 6, 7]
    assert list(bench.shard_universes(counts, 1, 0)) == [0, 1, 2]
    arrs = tuple(np.arange(18, dtype=np.float32) + k for k in range(7))
    sub, c = bench.select_universes(arrs, counts, [0, 2])
    assert list(c) == [5, 7] and sub[0].tolist() == list(range(5)) + list(range(11, 18))
