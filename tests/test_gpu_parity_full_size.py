"""GPU step against the oracle at the sizes the benchmark runs, with the benchmark's seeds.

The smaller parity cases (tests/test_gpu_parity.py) stop at a few tens of thousands of
bodies; these reach the tree depths, stack depths and work-item counts of the benchmarked
workloads:

* the 1,048,576-body Plummer sphere (vote width 64, two steps so that the second one
  applies the leapfrog velocity correction of calculateforce.cl:174-181): the default list
  walk; the per-visit walk with a 64-entry stack, which walks trees deeper than 9 levels
  with the per-level walk (calculateforce.cl:99-186) in every group; and the list walk with
  a 64-cell stack, which overflows for part of the groups and restarts them on the
  per-level walk;
* the ensemble of 256 Plummer universes, N per universe log-uniform in [1024, 65536]
  (3.59M bodies; 64-body work items that never straddle a universe);
* the disc with a central point mass and a Plummer halo in precise mode (Kahan-compensated
  updates, FP64 extent and root centre of mass), at 1,048,576 bodies: the same generator
  as the 4,194,304-body workload, a quarter of its bodies, so that the oracle's serial
  tree stages stay within seconds.

Each case asserts the same interaction count, the same depth-first order and the same
maximum depth as the oracle, and accelerations within 1e-4 relative per body (the
hardware inverse square root against the oracle's correctly rounded 1/sqrt).
"""
import numpy as np
import pytest

from helpers import KEYS, acc_rel, gpu_sim, oracle_for

pytestmark = pytest.mark.gpu

ACC_REL_MAX = 1e-4
ACC_REL_MEDIAN = 2e-6
SEED = 2024                  # bench.py's default seed


def _compare(g, o_state, o_sorted, o_inter, o_depth, where):
    st = g.stats()
    assert st["status"] == 0, where
    assert st["interactions"] == o_inter, (where, st["interactions"], o_inter)
    assert st["max_depth"] == o_depth, (where, st["max_depth"], o_depth)
    np.testing.assert_array_equal(g.tree()["sorted"], o_sorted, err_msg=where)
    gs = g.read()
    rel, _ = acc_rel(gs, o_state)
    assert rel.max() <= ACC_REL_MAX, (where, rel.max(), int(np.argmax(rel)))
    assert np.median(rel) <= ACC_REL_MEDIAN, (where, np.median(rel))
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        scale = max(1.0, float(np.abs(o_state[k]).max()))
        assert np.abs(gs[k] - o_state[k]).max() <= 1e-5 * scale, (where, k)
    return rel


@pytest.fixture(scope="module")
def plummer_1m():
    from nbh import universe as U
    n = 1 << 20
    arrs = U.PlummerUniverseGenerator(seed=SEED, a=1.0, M=1.0).arrays(n)
    o = oracle_for(n, theta=0.5, eps=0.05, dt=0.01, vote=64, fma=True)
    o.load(*arrs)
    assert o.step(2) == 0
    return arrs, o.state(), o.tree_arrays()["sorted"], o.interactions, o.maxdepth


@pytest.mark.parametrize("cap,force_list", [(0, 0), (64, 2), (64, 1)],
                         ids=["list-walk", "per-visit-per-level-walk", "list-walk-restarts"])
def test_plummer_1m_matches_oracle(plummer_1m, cap, force_list):
    arrs, o_state, o_sorted, o_inter, o_depth = plummer_1m
    g = gpu_sim(theta=0.5, eps=0.05, dt=0.01, vote_width=64, stack_cap=cap, force_list=force_list)
    g.load(*arrs)
    g.step(2)
    if cap == 64 and force_list == 2:
        # a 64-entry stack covers (64 - 8) / 7 + 1 = 9 levels; this tree is deeper, so every
        # group of the per-visit walk takes the per-level walk
        assert o_depth > 9
    _compare(g, o_state, o_sorted, o_inter, o_depth, "plummer 1M cap %d walk %d" % (cap, force_list))
    g.close()


def test_ensemble_256_matches_oracle_per_universe():
    import bench
    from nbh import universe as U
    counts = bench.ensemble_counts(256, SEED)
    parts = [U.PlummerUniverseGenerator(seed=SEED * 1000 + u, a=1.0, M=1.0).arrays(int(c))
             for u, c in enumerate(counts)]
    cat = [np.concatenate([p[k] for p in parts]) for k in range(7)]
    g = gpu_sim(theta=0.5, eps=0.05, dt=0.01, vote_width=64)
    g.load_batch(counts, *cat)
    g.step(1)
    gs = g.read()
    gsorted = g.tree()["sorted"]
    st = g.stats()
    total, depth, off = 0, 0, 0
    worst = 0.0
    for u, c in enumerate(counts):
        c = int(c)
        o = oracle_for(c, theta=0.5, eps=0.05, dt=0.01, vote=64, fma=True)
        o.load(*parts[u])
        assert o.step(1) == 0
        os_ = o.state()
        sub = {k: gs[k][off:off + c] for k in KEYS}
        rel, _ = acc_rel(sub, os_)
        worst = max(worst, float(rel.max()))
        assert rel.max() <= ACC_REL_MAX, (u, c, rel.max())
        np.testing.assert_array_equal(gsorted[off:off + c] - off, o.tree_arrays()["sorted"], err_msg="universe %d" % u)
        for k in ("x", "y", "z"):
            assert np.abs(sub[k] - os_[k]).max() <= 1e-5 * max(1.0, float(np.abs(os_[k]).max())), (u, k)
        total += o.interactions
        depth = max(depth, o.maxdepth)
        off += c
    assert off == int(counts.sum()) == g.n
    assert st["interactions"] == total
    assert st["max_depth"] == depth
    g.close()


def test_precise_disc_matches_oracle():
    from nbh import universe as U
    n = 1 << 20
    arrs = U.DiscGalaxyGenerator(seed=SEED, rd=1.0, zd=0.1, center_mass=0.1, halo_frac=0.1).arrays(n)
    o = oracle_for(n, theta=0.5, eps=0.05, dt=0.01, vote=64, fma=True, precise=True)
    o.load(*arrs)
    assert o.step(2) == 0
    g = gpu_sim(theta=0.5, eps=0.05, dt=0.01, vote_width=64, precise=True)
    g.load(*arrs)
    g.step(2)
    _compare(g, o.state(), o.tree_arrays()["sorted"], o.interactions, o.maxdepth, "precise disc 1M")
    g.close()
