"""Host-side logic that needs no GPU: the learned angle's training targets, the bench's
launch count, and the universe sharding helpers."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def test_theta_target_monotone_and_interpolated():
    from nbh import learned as LR
    grid = (0.4, 0.5, 0.6, 0.7)
    # rows = grid angles, columns = samples
    E = np.array([[1, 1, 1, 9],
                  [2, 5, 1, 9],
                  [9, 2, 1, 9],
                  [20, 20, 1, 9]], float)
    mono = np.exp(LR.theta_target(E, 3.0, grid=grid))
    loose = np.exp(LR.theta_target(E, 3.0, grid=grid, monotone=False))
    # sample 0: passes at 0.4 and 0.5, fails at 0.6 -> between 0.5 and 0.6 (log-interpolated)
    assert 0.5 < mono[0] < 0.6 and mono[0] == loose[0]
    # sample 1: fails at 0.5, passes at 0.6 by luck -> monotone stops below 0.5
    assert 0.4 < mono[1] < 0.5 and loose[1] > 0.6
    # sample 2: passes everywhere -> the largest grid angle
    assert abs(mono[2] - 0.7) < 1e-12
    # sample 3: fails everywhere -> the floor
    assert abs(mono[3] - 0.3) < 1e-12


def test_graph_launch_count_follows_the_build_schedule():
    import bench
    # bbox, link, summarize, sort, force, item order, integrate = 7, plus the build
    assert bench.graph_launches() == 7 + 3 + 4                 # five phases, bucketed
    assert bench.graph_launches(3, 1) == 7 + 1 + 2 * 4              # one lock phase, two bucketed passes
    assert bench.graph_launches(5, 2) == 7 + 5
    assert bench.graph_launches(1, 2) == 7 + 1
    assert bench.graph_launches(1, 1) == 7 + 1                 # one pass has no bucketed completion


def test_workload_shapes():
    import argparse
    import bench
    arrs, counts = bench.workload(argparse.Namespace(workload="ensemble", n=16, seed=5), 5)
    assert counts is not None and len(counts) == 16 and arrs[0].size == counts.sum()
    assert counts.min() >= 1024 and counts.max() <= 65536
    arrs, counts = bench.workload(argparse.Namespace(workload="ball", n=1000, seed=5), 5)
    assert counts is None and arrs[0].size == 1000
    r = np.sqrt(arrs[0] ** 2 + arrs[1] ** 2 + arrs[2] ** 2)
    assert r.max() <= 1.0 + 1e-6


def test_p99_ratio_interval_of_paired_errors():
    """The bootstrap interval of the learned-over-plain p99 ratio: identical arms give
    exactly 1; an arm scaled by 0.9 gives exactly 0.9 (every resample scales alike); and the
    interval of two unrelated arms holds their point ratio."""
    import numpy as np
    import bench
    rng = np.random.default_rng(3)
    ep = rng.lognormal(-7.0, 1.0, size=(8, 4096))
    assert bench._p99_ratio_interval(ep, ep, np) == [1.0, 1.0]
    lo, hi = bench._p99_ratio_interval(0.9 * ep, ep, np)
    assert abs(lo - 0.9) < 1e-12 and abs(hi - 0.9) < 1e-12
    el = rng.lognormal(-7.1, 0.9, size=(8, 4096))
    point = np.percentile(el, 99, axis=1).mean() / np.percentile(ep, 99, axis=1).mean()
    lo, hi = bench._p99_ratio_interval(el, ep, np)
    assert lo < point < hi and hi - lo < 0.2
