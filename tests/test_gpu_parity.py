"""GPU step through the C ABI against the oracle and the reference's golden fixtures.

Two arithmetic modes are checked:
* reference mode (vote width 16, rounded products, correctly rounded 1/sqrt): the GPU
  must equal the oracle bit for bit on every output, and the reference's own outputs
  within the reference's run-to-run spread (tests/test_oracle_golden.py);
* FMA mode (vote width 32, hardware rsqrt; the production path): same tree, same
  depth-first order and the same interaction count as the oracle; accelerations within
  relative 1e-4 per body (median 2e-6) of it, the difference being the ~2 ulp hardware
  inverse square root.  Vote width 64 (two bodies per lane) is checked the same way
  against the oracle's 64-body groups.
"""
import os

import numpy as np
import pytest

from helpers import GOLDEN, GOLDEN_FILES, KEYS, acc_rel, assert_same_tree, ball, gpu_sim, oracle_for, plummer

pytestmark = pytest.mark.gpu

FMA_ACC_REL_MAX = 1e-4
FMA_ACC_REL_MEDIAN = 2e-6


def _ref_mode_pair(G, vote=16):
    import nbh
    n = G["x0"].size
    g = gpu_sim(theta2=float(G["theta2"]), eps2=float(G["eps2"]), dt=float(G["dt"]), vote_width=vote,
                arith=nbh.NBH_ARITH_REFERENCE)
    args = (G["x0"], G["y0"], G["z0"], G["vx0"], G["vy0"], G["vz0"], G["m"])
    g.load(*args)
    o = oracle_for(n, theta2=float(G["theta2"]), eps2=float(G["eps2"]), dt=float(G["dt"]), vote=vote, fma=False)
    o.load(*args)
    return g, o


@pytest.mark.parametrize("path", GOLDEN_FILES, ids=[os.path.basename(f)[:-4] for f in GOLDEN_FILES])
def test_reference_mode_bit_exact_vs_oracle_and_golden(path):
    G = np.load(path)
    g, o = _ref_mode_pair(G)
    for s in range(int(G["steps"])):
        g.step()
        assert o.step() == 0
        gs, os_ = g.read(), o.state()
        for k in KEYS:
            np.testing.assert_array_equal(gs[k], os_[k], err_msg="%s step %d" % (k, s))
        # and the reference's own outputs within its run-to-run spread
        ref = {k: G[k][s] for k in KEYS}
        rel, scale_rel = acc_rel(gs, ref)
        assert rel.max() <= 5e-5 and np.median(rel) <= 1e-6 and scale_rel <= 2e-6
    t = g.tree()
    np.testing.assert_array_equal(t["sorted"], G["sorted"])
    st = g.stats()
    assert st["max_depth"] == int(G["maxdepth"])
    assert st["interactions"] == o.interactions


def test_reference_root_centre():
    """TestBoundingBox.testRoot (TestBoundingBox.java:205-247): 32768 bodies uniform in a
    cube of side 32768; after one step the tree root was centred at 0.5*(min+max) within
    1e-5; the first stage's root equals the host computation exactly here."""
    n = 2048 * 16
    rng = np.random.default_rng(3)
    x, y, z = (((rng.random(n) - 0.5) * n).astype(np.float32) for _ in range(3))
    m = np.full(n, 1.0 / n, np.float32)
    g = gpu_sim(theta=0.5, eps=0.05)
    g.load(x, y, z, None, None, None, m)
    o = oracle_for(n, theta=0.5, eps=0.05)
    o.load(x, y, z, None, None, None, m)
    o.bbox()
    g.step()
    t = g.tree()
    half = np.float32(0.5)
    assert t["radius"][0] == o.s.radius
    for k, arr in enumerate((x, y, z)):
        assert abs(float(half * (arr.min() + arr.max())) - float(o.tree_arrays()["xyz"[k]][o.nn])) < 1e-5


def test_fma_mode_matches_oracle_one_step():
    """16,384 bodies uniform in the unit ball, theta 0.5, eps 0.05, dt 0.025."""
    n = 16384
    arrs = ball(n, seed=5)
    g = gpu_sim(theta=0.5, eps=0.05, dt=0.025, vote_width=32)
    g.load(*arrs)
    o = oracle_for(n, theta=0.5, eps=0.05, dt=0.025, vote=32, fma=True)
    o.load(*arrs)
    g.step()
    o.step()
    gs, os_ = g.read(), o.state()
    st = g.stats()
    assert st["interactions"] == o.interactions
    assert st["max_depth"] == o.maxdepth
    np.testing.assert_array_equal(g.tree()["sorted"], o.tree_arrays()["sorted"])
    rel, _ = acc_rel(gs, os_)
    assert rel.max() <= FMA_ACC_REL_MAX, rel.max()
    assert np.median(rel) <= FMA_ACC_REL_MEDIAN, np.median(rel)
    for k in ("x", "y", "z"):
        assert np.abs(gs[k] - os_[k]).max() <= 1e-6


def test_fma_mode_ten_steps_positions():
    """The 16,384-body workload for its 10 steps: positions and velocities stay within
    1e-5 of the oracle's (relative to their extent)."""
    n = 16384
    arrs = ball(n, seed=6)
    g = gpu_sim(theta=0.5, eps=0.05, dt=0.025, vote_width=32)
    g.load(*arrs)
    o = oracle_for(n, theta=0.5, eps=0.05, dt=0.025, vote=32, fma=True)
    o.load(*arrs)
    g.step(10)
    o.step(10)
    gs, os_ = g.read(), o.state()
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        scale = np.abs(os_[k]).max()
        assert np.abs(gs[k] - os_[k]).max() <= 1e-5 * scale, k


@pytest.mark.parametrize("phases,buckets,top", [(5, 1, 0), (3, 1, 0), (5, 2, 0), (1, 2, 0), (5, 1, 2), (3, 2, 2),
                                               (5, 1, 3), (3, 2, 3)],
                         ids=["five-bucketed", "two-pass-bucketed", "five-lock", "one-pass",
                              "five-bucketed-global-first-phase", "three-lock-global-first-phase",
                              "five-bucketed-eight-blocks", "three-lock-eight-blocks"])
def test_tree_matches_oracle_and_invariants(phases, buckets, top):
    """Same octree as the oracle (slot by slot), every body in exactly one slot, body
    counts add up, root mass = total mass, centres of mass equal the oracle's bit for bit
    (same summation order) -- under every build schedule, with the first phase built in
    shared memory (one block per universe, the default at this size, or eight) or through the
    global locks."""
    n = 20000
    arrs = plummer(n, seed=9)
    g = gpu_sim(theta=0.5, eps=0.05, dt=0.01, vote_width=32, build_phases=phases, build_buckets=buckets,
                top_phase=top)
    g.load(*arrs)
    g.step()
    o = oracle_for(n, theta=0.5, eps=0.05, dt=0.01, vote=32, fma=True)
    o.load(*arrs)
    o.step()
    gt, ot = g.tree(), o.tree_arrays()
    nn = gt["nnodes"]
    cells = assert_same_tree(gt, ot, n, nn, o.nn)
    assert cells == nn + 1 - gt["bottom"] == o.nn + 1 - ot["bottom"]
    used = gt["child"][gt["bottom"] - n:]
    bodies = used[(used >= 0) & (used < n)]
    assert bodies.size == n and np.unique(bodies).size == n
    cnt = gt["count"]
    for c in range(gt["bottom"], nn + 1):
        ch = used[c - gt["bottom"]]
        tot = sum(1 if 0 <= v < n else (cnt[v - n] if v >= n else 0) for v in ch)
        assert tot == cnt[c - n]
        assert (np.diff((ch >= 0).astype(int)) <= 0).all(), "children not compacted"
    assert cnt[nn - n] == n
    root = gt["node4"][nn]
    assert abs(float(root[3]) - float(arrs[6].astype(np.float64).sum())) <= 1e-5
    assert root[3] == ot["m"][o.nn]
    assert root[0] == ot["x"][o.nn] and root[1] == ot["y"][o.nn] and root[2] == ot["z"][o.nn]


def _reachable_bodies(t, n, roots=None):
    """Bodies reachable from the root(s) through the child slots, level by level."""
    child, out = t["child"], []
    front = np.array([t["nnodes"]]) if roots is None else np.asarray(roots)
    while front.size:
        ch = child[front - n].ravel()
        out.append(ch[(ch >= 0) & (ch < n)])
        front = ch[ch >= n]
    return np.concatenate(out)


def test_rebuilds_under_contention_hold_every_body_and_repeat():
    """1M-body Plummer sphere with dt = 0: every step rebuilds the same octree from the same
    positions.  Under every build schedule (one lock pass: all bodies contend at once; five
    lock phases; five phases with the bucketed completion; one lock phase with two bucketed
    passes; five bucketed phases with the first phase in one shared-memory block instead of
    the eight the default takes at this size) each rebuild reaches every body
    exactly once from the root, counts them all, and gives the same depth-first order and
    the same accelerations, bit for bit, as every other rebuild and schedule.  (Summarize
    used to decide from a cell's slots while the cell's own compaction rewrote them; in up to
    a third of the one-pass rebuilds that dropped a few bodies.)"""
    n = 1 << 20
    arrs = plummer(n, seed=1)
    ref = None
    for phases, buckets, steps, top in ((1, 2, 12, 0), (5, 2, 5, 0), (5, 1, 5, 0), (3, 1, 5, 0), (5, 1, 3, 1)):
        g = gpu_sim(theta=0.5, eps=0.05, dt=0.0, vote_width=64, build_phases=phases, build_buckets=buckets,
                    top_phase=top)
        g.load(*arrs)
        for s in range(steps):
            g.step()
            t = g.tree()
            where = "schedule %d/%d rebuild %d" % (phases, buckets, s)
            reach = _reachable_bodies(t, n)
            assert reach.size == n and np.unique(reach).size == n, where
            assert t["count"][t["nnodes"] - n] == n, where
            srt = t["sorted"]
            assert np.array_equal(np.sort(srt), np.arange(n)), where
            st = g.read()
            acc = np.stack([st["ax"], st["ay"], st["az"]])
            if ref is None:
                ref = (srt.copy(), acc)
            else:
                np.testing.assert_array_equal(srt, ref[0], err_msg=where)
                np.testing.assert_array_equal(acc, ref[1], err_msg=where)
        g.close()


def test_first_phase_falls_back_to_global_locks_when_shared_memory_is_full():
    """The first insertion phase (one body of every 256-body chunk) builds the top of the tree
    in shared memory, one block per universe or one per octant of the root, each holding about
    one cell per sampled body of the universe (2,112 here).  Here all 2,048 sampled bodies lie
    in one octant and come in close pairs (2^-17 of the extent apart), so each pair makes a
    chain of ~15 single-child cells and that octant needs ~13,700 cells: the block inserts its
    sample through the global locks instead, in both layouts.  The tree equals the oracle's slot by slot, and the
    step equals the one with the global first phase chosen from the start, bit for bit."""
    n = 2048 * 256
    rng = np.random.default_rng(11)
    x, y, z = (rng.uniform(-1.0, 1.0, n).astype(np.float32) for _ in range(3))
    m = np.full(n, 1.0 / n, np.float32)
    chunk = np.arange(n // 256)
    smp = chunk * 256 + ((7 * chunk) & 15)          # the first phase's body of each chunk
    x[smp], y[smp], z[smp] = np.abs(x[smp]), np.abs(y[smp]), np.abs(z[smp])   # one octant
    d = np.float32(2.0 ** -17)
    for k in range(0, smp.size, 2):                 # every second sample sits next to the one before
        a, b = smp[k], smp[k + 1]
        x[b], y[b], z[b] = x[a] + d, y[a], z[a]
    arrs = (x, y, z, None, None, None, m)
    outs = []
    for top in (1, 3, 2):
        g = gpu_sim(theta=0.5, eps=0.05, dt=0.01, vote_width=64, top_phase=top)
        g.load(*arrs)
        g.step()
        assert g.stats()["status"] == 0
        outs.append((g.tree(), g.read(), g.stats()["interactions"]))
        g.close()
    o = oracle_for(n, theta=0.5, eps=0.05, dt=0.01, vote=64, fma=True)
    o.load(*arrs)
    assert o.tree() == 0
    gt, ot = outs[0][0], o.tree_arrays()
    assert assert_same_tree(gt, ot, n, gt["nnodes"], o.nn) == gt["nnodes"] + 1 - gt["bottom"]
    np.testing.assert_array_equal(gt["sorted"], ot["sorted"])
    for other in outs[1:]:
        np.testing.assert_array_equal(gt["sorted"], other[0]["sorted"])
        assert outs[0][2] == other[2]
        for k in KEYS:
            np.testing.assert_array_equal(outs[0][1][k], other[1][k])


def test_batch_of_universes_matches_oracle_per_universe():
    """Several uneven universes in one sim: each equals the oracle run on it alone."""
    import nbh
    from nbh import universe as U
    counts = [1024, 33, 5000, 1, 12000, 2048]
    parts = [U.PlummerUniverseGenerator(seed=40 + i).arrays(c) for i, c in enumerate(counts)]
    cat = [np.concatenate([p[k] for p in parts]) for k in range(7)]
    g = gpu_sim(theta=0.5, eps=0.05, dt=0.01, vote_width=32)
    g.load_batch(counts, *cat)
    g.step(3)
    gs = g.read()
    total_inter = 0
    off = 0
    for i, c in enumerate(counts):
        o = oracle_for(c, theta=0.5, eps=0.05, dt=0.01, vote=32, fma=True)
        o.load(*parts[i])
        o.step(3)
        os_ = o.state()
        sl = slice(off, off + c)
        sub = {k: gs[k][sl] for k in KEYS}
        rel, _ = acc_rel(sub, os_)
        assert rel.max() <= FMA_ACC_REL_MAX, (i, rel.max())
        for k in ("x", "y", "z"):
            assert np.abs(sub[k] - os_[k]).max() <= 1e-5 * max(1.0, np.abs(os_[k]).max())
        total_inter += o.interactions
        off += c
    assert g.stats()["interactions"] == total_inter
    assert isinstance(nbh.Simulation, type)


@pytest.mark.parametrize("vote,n", [(64, 20000), (64, 64), (64, 65), (64, 1), (128, 20000), (128, 129), (128, 127)])
def test_vote64_matches_oracle_one_step(vote, n):
    """Vote widths 64 and 128 (two or four bodies per lane): groups of that many consecutive
    sorted bodies, the last one ragged; same interactions, same depth-first order,
    accelerations within the FMA tolerance of the oracle's groups of the same size."""
    arrs = plummer(n, seed=21)
    g = gpu_sim(theta=0.5, eps=0.05, dt=0.01, vote_width=vote)
    g.load(*arrs)
    o = oracle_for(n, theta=0.5, eps=0.05, dt=0.01, vote=vote, fma=True)
    o.load(*arrs)
    g.step(2)
    o.step(2)
    gs, os_ = g.read(), o.state()
    st = g.stats()
    assert st["interactions"] == o.interactions
    np.testing.assert_array_equal(g.tree()["sorted"], o.tree_arrays()["sorted"])
    rel, _ = acc_rel(gs, os_)
    assert rel.max() <= FMA_ACC_REL_MAX, rel.max()
    for k in ("x", "y", "z"):
        assert np.abs(gs[k] - os_[k]).max() <= 1e-5 * max(1.0, np.abs(os_[k]).max())


@pytest.mark.parametrize("vote,force_list,cap,theta",
                         [(64, 1, 256, 0.5), (64, 2, 256, 0.5), (64, 1, 64, 0.5), (64, 1, 256, 0.15),
                          (64, 1, 64, 0.15), (32, 1, 256, 0.5), (32, 2, 256, 0.5), (32, 1, 64, 0.15),
                          (128, 1, 256, 0.5), (128, 1, 64, 0.15)],
                         ids=["list-walk", "per-visit-walk", "list-walk-overflow-restarts", "list-walk-small-angle",
                              "list-walk-small-angle-overflow", "list-walk-32", "per-visit-walk-32",
                              "list-walk-32-small-angle-overflow", "list-walk-128", "list-walk-128-small-angle-overflow"])
def test_list_walk_matches_oracle(vote, force_list, cap, theta):
    """The whole-warp walks (vote widths 32, 64, 128) in both forms: the lane-parallel list
    walk (box and representative decide most votes, accepted records evaluated from a
    shared-memory list) and one child at a time.  Both take the oracle's votes: the same
    interactions and depth-first order, accelerations within the FMA tolerance.  A 64-cell
    stack overflows for part of the groups (up to ~80 pending cells at theta 0.5, ~140 at
    0.15 on this sphere at width 64), which restart on the per-level walk, with the same
    result."""
    n = 20000
    arrs = plummer(n, seed=91)
    g = gpu_sim(theta=theta, eps=0.05, dt=0.01, vote_width=vote, force_list=force_list, stack_cap=cap)
    g.load(*arrs)
    o = oracle_for(n, theta=theta, eps=0.05, dt=0.01, vote=vote, fma=True)
    o.load(*arrs)
    g.step(2)
    o.step(2)
    gs, os_ = g.read(), o.state()
    assert g.stats()["interactions"] == o.interactions
    np.testing.assert_array_equal(g.tree()["sorted"], o.tree_arrays()["sorted"])
    rel, _ = acc_rel(gs, os_)
    assert rel.max() <= FMA_ACC_REL_MAX, rel.max()
    assert np.median(rel) <= FMA_ACC_REL_MEDIAN, np.median(rel)


def test_list_walk_and_per_visit_walk_agree_at_1m():
    """1M-body Plummer sphere: the list walk and the per-visit walk accept the same nodes (the
    same interaction count) and their sums differ only by rounding order."""
    n = 1 << 20
    arrs = plummer(n, seed=2024)
    acc, inter = {}, {}
    for fl in (1, 2):
        g = gpu_sim(theta=0.5, eps=0.05, dt=0.01, vote_width=64, force_list=fl)
        g.load(*arrs)
        g.step(1)
        r = g.read()
        acc[fl] = np.stack([r["ax"], r["ay"], r["az"]]).astype(np.float64)
        inter[fl] = g.stats()["interactions"]
        g.close()
    assert inter[1] == inter[2]
    rel = np.linalg.norm(acc[1] - acc[2], axis=0) / np.linalg.norm(acc[2], axis=0)
    assert rel.max() <= 1e-4 and np.median(rel) <= 2e-6, (rel.max(), np.median(rel))


@pytest.mark.parametrize("vote", [64, 128])
def test_vote64_batch_of_universes(vote):
    """Vote widths 64 and 128 over uneven universes: items never straddle a universe
    boundary."""
    from nbh import universe as U
    counts = [1024, 33, 5000, 1, 64, 65, 127, 129]
    parts = [U.PlummerUniverseGenerator(seed=60 + i).arrays(c) for i, c in enumerate(counts)]
    cat = [np.concatenate([p[k] for p in parts]) for k in range(7)]
    g = gpu_sim(theta=0.5, eps=0.05, dt=0.01, vote_width=vote)
    g.load_batch(counts, *cat)
    g.step(2)
    gs = g.read()
    total, off = 0, 0
    for i, c in enumerate(counts):
        o = oracle_for(c, theta=0.5, eps=0.05, dt=0.01, vote=vote, fma=True)
        o.load(*parts[i])
        o.step(2)
        rel, _ = acc_rel({k: gs[k][off:off + c] for k in KEYS}, o.state())
        assert rel.max() <= FMA_ACC_REL_MAX, (i, rel.max())
        total += o.interactions
        off += c
    assert g.stats()["interactions"] == total


def test_graph_and_eager_paths_identical():
    n = 8192
    arrs = plummer(n, seed=2)
    outs = []
    for use_graph, timing in ((True, False), (False, False), (False, True)):
        g = gpu_sim(theta=0.5, eps=0.05, dt=0.01, use_graph=use_graph, stage_timing=timing)
        g.load(*arrs)
        g.step(4)
        outs.append(g.read())
        if timing:
            st = g.stats()
            assert st["ms_force"] > 0 and st["ms_step"] >= st["ms_force"]
    for o in outs[1:]:
        for k in KEYS:
            np.testing.assert_array_equal(outs[0][k], o[k])


def test_precise_mode_matches_oracle():
    """Kahan-compensated updates and FP64 root/extent, GPU vs oracle in the same mode."""
    n = 8192
    arrs = plummer(n, seed=12)
    g = gpu_sim(theta=0.5, eps=0.05, dt=0.01, precise=True, vote_width=32)
    g.load(*arrs)
    o = oracle_for(n, theta=0.5, eps=0.05, dt=0.01, vote=32, fma=True, precise=True)
    o.load(*arrs)
    g.step(5)
    o.step(5)
    gs, os_ = g.read(), o.state()
    rel, _ = acc_rel(gs, os_)
    assert rel.max() <= FMA_ACC_REL_MAX
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        assert np.abs(gs[k] - os_[k]).max() <= 1e-5 * np.abs(os_[k]).max()


def test_precise_mode_list_walk_option_keeps_the_interactions_and_the_error():
    """Precise mode keeps the per-visit walk (the oracle's depth-first order of accumulation)
    unless force_list = 1 asks for the list walk.  On a disc with a central point mass and a
    halo (262,144 bodies, the 4M workload's generator) the list walk accepts the same nodes,
    and its force error against the FP64 direct sum on sampled bodies has the same p99 and
    median; the two sums differ by rounding order only (the central mass, whose acceleration
    nearly cancels, is where they differ most)."""
    import oracle as O
    from nbh import universe as U
    n = 1 << 18
    arrs = U.DiscGalaxyGenerator(seed=31, rd=1.0, zd=0.1, center_mass=0.1, halo_frac=0.1).arrays(n)
    idx = np.sort(np.random.default_rng(3).choice(n, 4096, replace=False)).astype(np.int32)
    res = {}
    for fl in (2, 1):
        g = gpu_sim(theta=0.5, eps=0.05, dt=0.01, vote_width=64, precise=True, force_list=fl)
        g.load(*arrs)
        ref = g.direct_f64(idx)
        g.step(1)
        st = g.read()
        err = O.rel_force_error(st["ax"][idx], st["ay"][idx], st["az"][idx], *ref)
        res[fl] = (g.stats()["interactions"], g.tree()["sorted"], st, err)
        g.close()
    assert res[1][0] == res[2][0]
    np.testing.assert_array_equal(res[1][1], res[2][1])
    e1, e2 = res[1][3], res[2][3]
    assert abs(np.percentile(e1, 99) / np.percentile(e2, 99) - 1) <= 1e-3
    assert abs(np.median(e1) / np.median(e2) - 1) <= 1e-3
    rel, _ = acc_rel(res[1][2], res[2][2])
    assert np.median(rel) <= FMA_ACC_REL_MEDIAN, np.median(rel)


def test_precise_mode_keeps_increments_below_an_ulp():
    """Two light bodies at x = +-1000 drifting at 1e-3 with dt = 1e-3: each step moves them
    1e-6, below half an FP32 ulp at 1000 (6.1e-5), so plain updates never move them while
    the Kahan-compensated ones (precise mode) advance them by 1000 steps * 1e-6 = 1e-3."""
    x = np.array([1000.0, -1000.0], np.float32)
    z0 = np.zeros(2, np.float32)
    vx = np.array([1e-3, -1e-3], np.float32)
    m = np.full(2, 1e-12, np.float32)            # forces ~1e-19: negligible
    out = {}
    for precise in (False, True):
        g = gpu_sim(theta=0.5, eps=0.05, dt=1e-3, precise=precise)
        g.load(x, z0, z0, vx, z0, z0, m)
        g.step(1000)
        out[precise] = g.read()["x"].astype(np.float64)
        g.close()
    np.testing.assert_array_equal(out[False], x.astype(np.float64))
    ulp = np.spacing(np.float32(1000.0))
    np.testing.assert_allclose(out[True], [1000.0 + 1e-3, -1000.0 - 1e-3], rtol=0, atol=float(ulp))


def test_pinned_host_arrays_match_the_staged_path():
    """nbh_write / nbh_read with pinned host arrays (read and written in place by one kernel)
    give exactly what pageable arrays (staged copies) give."""
    torch = pytest.importorskip("torch")
    n = 30000
    arrs = plummer(n, seed=91)
    keys = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az")
    res = {}
    for pinned in (False, True):
        g = gpu_sim(theta=0.5, eps=0.05, dt=0.01)
        g.load(*arrs)
        g.step(2)
        st = g.read()
        if pinned:
            hin = {k: torch.empty(n, dtype=torch.float32, pin_memory=True).numpy() for k in keys}
            hout = {k: torch.empty(n, dtype=torch.float32, pin_memory=True).numpy() for k in keys}
        else:
            hin = {k: np.empty(n, np.float32) for k in keys}
            hout = {k: np.empty(n, np.float32) for k in keys}
        for k in keys:
            hin[k][:] = st[k] * np.float32(1.0 + 1e-3)    # a modified state to write back
        g.write(*[hin[k] for k in keys])
        g.step(1)
        g.read_into(*[hout[k] for k in keys])
        res[pinned] = {k: hout[k].copy() for k in keys}
        g.close()
    for k in keys:
        np.testing.assert_array_equal(res[True][k], res[False][k])


def test_step_io_equals_write_step_read():
    """nbh_step_io (write, steps, read, one wait) gives exactly what nbh_write + nbh_step +
    nbh_read give, with pinned and with pageable arrays, and with only one of its two parts;
    a write of positions only keeps velocities and accelerations."""
    torch = pytest.importorskip("torch")
    n = 30000
    arrs = plummer(n, seed=92)
    keys = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az")

    def fresh():
        g = gpu_sim(theta=0.5, eps=0.05, dt=0.01)
        g.load(*arrs)
        g.step(2)
        return g
    g = fresh()
    st = g.read()
    hin = {k: st[k] * np.float32(1.0 + 1e-3) for k in keys}
    g.write(*[hin[k] for k in keys])
    g.step(3)
    want = g.read()
    g.close()
    for pinned in (False, True):
        if pinned:
            src = {k: torch.empty(n, dtype=torch.float32, pin_memory=True).numpy() for k in keys}
            out = {k: torch.empty(n, dtype=torch.float32, pin_memory=True).numpy() for k in keys}
        else:
            src = {k: np.empty(n, np.float32) for k in keys}
            out = {k: np.empty(n, np.float32) for k in keys}
        for k in keys:
            src[k][:] = hin[k]
        g = fresh()
        g.step_io(3, write=src, read=out)
        for k in keys:
            np.testing.assert_array_equal(out[k], want[k], err_msg="%s pinned=%s" % (k, pinned))
        g.close()
    # velocities and accelerations alone (pinned: they go up beside the tree stages)
    vin = {k: torch.empty(n, dtype=torch.float32, pin_memory=True).numpy() for k in keys[3:]}
    for k in keys[3:]:
        vin[k][:] = hin[k]
    g = fresh()
    g.write(None, None, None, *[hin[k] for k in keys[3:]])
    g.step(2)
    want_v = g.read()
    g.close()
    g = fresh()
    g.step_io(2, write=vin)
    got_v = g.read()
    for k in keys:
        np.testing.assert_array_equal(got_v[k], want_v[k], err_msg="velocity-only write: %s" % k)
    g.close()
    # write only, then read only; positions only leave the rest as they were
    g = fresh()
    g.step_io(0, write={k: hin[k] for k in keys})
    g.step_io(3)
    part = {k: np.empty(n, np.float32) for k in ("x", "vz")}
    g.step_io(0, read=part)
    np.testing.assert_array_equal(part["x"], want["x"])
    np.testing.assert_array_equal(part["vz"], want["vz"])
    before = g.read()
    g.step_io(0, write={"x": hin["x"], "y": hin["y"], "z": hin["z"]})
    after = g.read()
    np.testing.assert_array_equal(after["x"], hin["x"])
    for k in ("vx", "vy", "vz", "ax", "ay", "az"):
        np.testing.assert_array_equal(after[k], before[k])
    import nbh
    from nbh import _lib as L
    with pytest.raises(nbh.NbhError) as ei:
        g.step_io(1, write={"x": hin["x"]})           # positions need x, y and z
    assert ei.value.code == L.NBH_ERR_INVALID
    g.close()


def test_batch_rebuilds_under_contention_hold_every_body_and_repeat():
    """A batch of 192 Plummer universes (1 to 40,000 bodies, 625,654 in all) with dt = 0, built in
    one lock pass (every universe's bodies contend in its top levels at once), with the
    default schedule and with the two-pass bucketed one: every rebuild reaches every body
    once from its own universe's root,
    and repeats the depth-first order and the accelerations bit for bit."""
    from nbh import universe as U
    rng = np.random.default_rng(11)
    counts = np.exp(rng.uniform(0.0, np.log(40000), 192)).astype(np.int32)
    counts[:3] = (1, 2, 40000)
    parts = [U.PlummerUniverseGenerator(seed=300 + i).arrays(int(c)) for i, c in enumerate(counts)]
    cat = [np.concatenate([p[k] for p in parts]) for k in range(7)]
    n = int(counts.sum())
    off = np.concatenate([[0], np.cumsum(counts)])
    ref = None
    for phases, buckets in ((1, 2), (5, 1), (3, 1)):
        g = gpu_sim(theta=0.5, eps=0.05, dt=0.0, vote_width=64, build_phases=phases, build_buckets=buckets)
        g.load_batch(counts, *cat)
        for s in range(4):
            g.step()
            t = g.tree()
            where = "schedule %d/%d rebuild %d" % (phases, buckets, s)
            reach = _reachable_bodies(t, n, t["roots"])
            assert reach.size == n and np.unique(reach).size == n, where
            for u in (0, 1, 2, 100):      # each body hangs below its own universe's root
                ru = _reachable_bodies(t, n, [t["roots"][u]])
                assert np.array_equal(np.sort(ru), np.arange(off[u], off[u + 1])), (where, u)
            st = g.read()
            acc = np.stack([st["ax"], st["ay"], st["az"]])
            if ref is None:
                ref = (t["sorted"].copy(), acc)
            else:
                np.testing.assert_array_equal(t["sorted"], ref[0], err_msg=where)
                np.testing.assert_array_equal(acc, ref[1], err_msg=where)
        g.close()


def test_long_run_keeps_every_tree_whole():
    """200 steps of a moving 1M-body Plummer sphere (autotuned geometry, default schedule):
    every 50 steps the tree reaches each body once from the root, the depth-first order is a
    permutation, the state is finite and the step reports no error."""
    n = 1 << 20
    g = gpu_sim(theta=0.5, eps=0.05, dt=0.01)
    g.load(*plummer(n, seed=3))
    g.autotune()
    for s in range(4):
        g.step(50)
        t = g.tree()
        reach = _reachable_bodies(t, n)
        assert reach.size == n and np.unique(reach).size == n, s
        assert np.array_equal(np.sort(t["sorted"]), np.arange(n)), s
        st = g.read()
        assert all(np.isfinite(st[k]).all() for k in KEYS), s
        assert g.stats()["status"] == 0
    g.close()


def test_long_run_of_a_batch_with_the_first_phase_in_shared_memory():
    """200 steps of 64 moving Plummer universes (1K-64K bodies) with the first insertion
    phase built in shared memory every step: every 50 steps each universe's tree reaches
    each of its bodies once from its root, the depth-first order is a permutation inside
    each universe's range, the state is finite and no step reports an error."""
    import bench
    from nbh import universe as U
    counts = bench.ensemble_counts(64, 7)
    parts = [U.PlummerUniverseGenerator(seed=700 + u).arrays(int(c)) for u, c in enumerate(counts)]
    cat = [np.concatenate([p[k] for p in parts]) for k in range(7)]
    n = int(counts.sum())
    offs = np.concatenate([[0], np.cumsum(counts)])
    g = gpu_sim(theta=0.5, eps=0.05, dt=0.01, top_phase=1)
    g.load_batch(counts, *cat)
    for s in range(4):
        g.step(50)
        assert g.stats()["status"] == 0
        t = g.tree()
        roots = t["nnodes"] - np.arange(counts.size)
        reach = _reachable_bodies(t, n, roots)
        assert reach.size == n and np.unique(reach).size == n, s
        srt = t["sorted"]
        for u in range(counts.size):
            seg = srt[offs[u]:offs[u + 1]]
            assert np.array_equal(np.sort(seg), np.arange(offs[u], offs[u + 1])), (s, u)
        st = g.read()
        assert all(np.isfinite(st[k]).all() for k in KEYS), s
    g.close()


def test_massless_tracers_match_oracle():
    """A quarter of the bodies carry no mass (tracers).  Cells holding only tracers have no
    defined centre of mass (0/0, as in the reference's summarize), never pass the opening
    test and are always opened; the tracers still feel the massive bodies.  Same interactions
    and forces as the oracle."""
    n = 20000
    arrs = list(plummer(n, seed=93))
    m = arrs[6].copy()
    m[::4] = 0.0
    arrs[6] = m
    g = gpu_sim(theta=0.5, eps=0.05, dt=0.01, vote_width=32)
    g.load(*arrs)
    o = oracle_for(n, theta=0.5, eps=0.05, dt=0.01, vote=32, fma=True)
    o.load(*arrs)
    g.step(2)
    o.step(2)
    gs = g.read()
    assert g.stats()["status"] == 0
    assert g.stats()["interactions"] == o.interactions
    for k in ("ax", "ay", "az", "x", "y", "z"):
        assert np.isfinite(gs[k]).all(), k
    rel, _ = acc_rel(gs, o.state())
    assert rel.max() <= FMA_ACC_REL_MAX, rel.max()


def test_direct_f64_matches_oracle():
    import oracle as O
    n = 30000
    arrs = plummer(n, seed=21)
    g = gpu_sim(theta=0.5, eps=0.05)
    g.load(*arrs)
    idx = np.random.default_rng(0).choice(n, 97, replace=False).astype(np.int32)
    ga = g.direct_f64(idx)
    oa = O.direct_f64(arrs[0], arrs[1], arrs[2], arrs[6], 0.05, idx)
    for a, b in zip(ga, oa):
        np.testing.assert_allclose(a, b, rtol=1e-10, atol=1e-12)


def test_force_error_vs_fp64_plummer():
    """theta 0.5 on a 65,536-body Plummer sphere: median and p99 relative force error
    against the FP64 direct sum on 1,024 sampled bodies."""
    import oracle as O
    n = 65536
    arrs = plummer(n, seed=33)
    g = gpu_sim(theta=0.5, eps=0.05, dt=0.01)
    g.load(*arrs)
    g.step()
    gs = g.read()
    idx = np.random.default_rng(1).choice(n, 1024, replace=False).astype(np.int32)
    # accelerations of step 1 belong to the positions before the drift
    g2 = gpu_sim(theta=0.5, eps=0.05, dt=0.01)
    g2.load(*arrs)
    ref = g2.direct_f64(idx)
    err = O.rel_force_error(gs["ax"][idx], gs["ay"][idx], gs["az"][idx], *ref)
    assert np.median(err) < 2e-3, np.median(err)
    assert np.percentile(err, 99) < 2e-2, np.percentile(err, 99)


def test_export_float4_matches_read():
    import torch
    n = 5000
    arrs = plummer(n, seed=4)
    g = gpu_sim()
    g.load(*arrs)
    g.step(2)
    pos4 = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    vel4 = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    g.export_float4(pos4.data_ptr(), vel4.data_ptr())
    st = g.read()
    p, v = pos4.cpu().numpy(), vel4.cpu().numpy()
    np.testing.assert_array_equal(p[:, 0], st["x"])
    np.testing.assert_array_equal(v[:, 2], st["vz"])
    assert (p[:, 3] == 1).all() and (v[:, 3] == 1).all()


def test_write_resumes_from_checkpoint():
    """Read the state after 3 steps, write it into a fresh sim whose step counter is
    advanced the same way: the next steps agree bit for bit."""
    n = 6000
    arrs = plummer(n, seed=8)
    a = gpu_sim(dt=0.01)
    a.load(*arrs)
    a.step(3)
    ck = a.read()
    b = gpu_sim(dt=0.01)
    b.load(*arrs)
    b.step(3)                          # same step counter as a
    b.write(*[ck[k] for k in KEYS])
    a.step(2)
    b.step(2)
    ra, rb = a.read(), b.read()
    for k in KEYS:
        np.testing.assert_array_equal(ra[k], rb[k])
