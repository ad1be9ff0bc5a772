"""Launch-geometry autotuner and the run-time force geometry on GB300: every geometry gives
the same results, and the tuner leaves the simulation state as it found it."""
import numpy as np
import pytest

from helpers import KEYS, acc_rel, gpu_sim, oracle_for, plummer

pytestmark = pytest.mark.gpu


def test_autotune_choice_changes_no_result():
    n = 20000
    arrs = plummer(n, seed=81)
    a = gpu_sim(theta=0.5, eps=0.05, dt=0.01)
    b = gpu_sim(theta=0.5, eps=0.05, dt=0.01)
    a.load(*arrs)
    b.load(*arrs)
    a.step(2)
    b.step(2)
    before = b.stats()
    t = b.autotune()
    after = b.stats()
    assert after["steps"] == before["steps"] and after["max_depth"] == before["max_depth"]
    assert t["force_threads"] in (64, 128, 256) and 64 <= t["stack_cap"] <= 256 and t["build_phases"] in (1, 3, 5)
    assert t["max_depth"] == before["max_depth"]
    assert (t["stack_cap"] - 8) // 7 + 1 >= t["max_depth"] or t["stack_cap"] == 256
    assert any(tr["kind"] == "force" for tr in t["trials"]) and any(tr["kind"] == "tree" for tr in t["trials"])
    assert t["ms_force"] <= t["ms_force_before"] + 1e-6 and t["ms_tree"] <= t["ms_tree_before"] + 1e-6
    # state untouched by the tuning launches
    sa, sb = a.read(), b.read()
    for k in KEYS:
        np.testing.assert_array_equal(sa[k], sb[k])
    a.step(3)
    b.step(3)
    sa, sb = a.read(), b.read()
    for k in KEYS:
        np.testing.assert_array_equal(sa[k], sb[k])
    assert a.stats()["interactions"] == b.stats()["interactions"]


@pytest.mark.parametrize("vote,threads,cap", [(64, 64, 64), (64, 256, 96), (32, 64, 128), (16, 256, 64)])
def test_force_geometries_match_oracle(vote, threads, cap):
    """Block sizes and stack capacities, including a 64-entry stack that sends a 14-level
    tree through the per-level walk (fast path only up to 9 levels)."""
    n = 20000
    arrs = plummer(n, seed=82)
    g = gpu_sim(theta=0.5, eps=0.05, dt=0.01, vote_width=vote, force_threads=threads, stack_cap=cap)
    g.load(*arrs)
    o = oracle_for(n, theta=0.5, eps=0.05, dt=0.01, vote=vote, fma=True)
    o.load(*arrs)
    g.step(2)
    o.step(2)
    assert g.stats()["interactions"] == o.interactions
    rel, _ = acc_rel(g.read(), o.state())
    assert rel.max() <= 1e-4, rel.max()


@pytest.mark.parametrize("phases,buckets", [(1, 2), (5, 2), (3, 1), (5, 1)])
def test_phase_schedules_give_the_same_tree(phases, buckets):
    n = 30000
    arrs = plummer(n, seed=83)
    a = gpu_sim(theta=0.5, eps=0.05, dt=0.01, build_phases=phases, build_buckets=buckets)
    b = gpu_sim(theta=0.5, eps=0.05, dt=0.01, build_phases=3, build_buckets=2)
    a.load(*arrs)
    b.load(*arrs)
    a.step(2)
    b.step(2)
    np.testing.assert_array_equal(a.tree()["sorted"], b.tree()["sorted"])
    sa, sb = a.read(), b.read()
    for k in KEYS:
        np.testing.assert_array_equal(sa[k], sb[k])


def test_vote_tuning_picks_a_width_and_stays_parity_clean():
    """NBH_TUNE_VOTE times vote widths 32 and 64; the chosen width then matches the oracle's
    groups of that size."""
    n = 20000
    arrs = plummer(n, seed=84)
    g = gpu_sim(theta=0.5, eps=0.05, dt=0.01)
    g.load(*arrs)
    g.step(1)
    t = g.autotune(vote=True)
    assert t["vote_width"] in (16, 32, 64, 128)
    assert {tr["vote"] for tr in t["trials"] if tr["kind"] == "force"} == {16, 32, 64, 128}
    before = g.read()
    o = oracle_for(n, theta=0.5, eps=0.05, dt=0.01, vote=t["vote_width"], fma=True)
    o.load(*[before[k] for k in ("x", "y", "z", "vx", "vy", "vz")], arrs[6])
    g.step(1)
    o.step(1)
    assert g.stats()["interactions"] == o.interactions
    rel, _ = acc_rel(g.read(), o.state())
    assert rel.max() <= 1e-4


def test_vote_tuning_refused_in_reference_arithmetic():
    import nbh
    g = gpu_sim(theta2=1.5, eps2=0.0025, dt=0.025, vote_width=16, arith=nbh.NBH_ARITH_REFERENCE)
    g.load(*plummer(4096, seed=85))
    with pytest.raises(nbh.NbhError):
        g.autotune(vote=True)


def test_bucketed_build_when_the_sample_misses_a_cluster():
    """An input order aliased with the sample lattice (in chunk c of 256 bodies the sample
    takes the offsets congruent to 7c mod 16): the sampled bodies are spread over a cube, the
    other 15 in 16 sit in a tiny ball the sample never reaches, so one slot's bucket holds
    almost every body (the large-bucket path, many levels deep).  The tree and the forces
    equal the lock-only build's."""
    n = 16 * 4096
    r = np.random.default_rng(86)
    pos = r.uniform(-1, 1, (n, 3)).astype(np.float32)
    i = np.arange(n)
    rest = ((i % 256) - 7 * (i // 256)) % 16 != 0
    pos[rest] = (np.float32(0.31) + r.normal(0, 1e-3, (int(rest.sum()), 3))).astype(np.float32)
    zero = np.zeros(n, np.float32)
    m = np.full(n, 1.0 / n, np.float32)
    arrs = (pos[:, 0].copy(), pos[:, 1].copy(), pos[:, 2].copy(), zero, zero, zero, m)
    out = {}
    for buckets in (1, 2):
        g = gpu_sim(theta=0.5, eps=0.05, dt=0.01, build_phases=5, build_buckets=buckets)
        g.load(*arrs)
        g.step(1)
        out[buckets] = (g.tree()["sorted"], g.read(), g.stats())
        g.close()
    np.testing.assert_array_equal(out[1][0], out[2][0])
    for k in KEYS:
        np.testing.assert_array_equal(out[1][1][k], out[2][1][k])
    assert out[1][2]["max_depth"] == out[2][2]["max_depth"] and out[1][2]["status"] == 0


def test_close_pairs_inside_the_sample_make_long_chains():
    """Close pairs whose both bodies fall in the build's 1/16 sample (offsets o and o + 16
    of a chunk, o on the sample lattice): the sample tree then holds long chains of cells
    with one cell child (~17 levels per pair), many more cells than sampled bodies.  Every
    build schedule -- one lock pass, five lock phases, five phases with the bucketed
    completion, one lock phase with two bucketed passes -- gives the same tree and forces,
    with every body reachable once from the root."""
    n = 16 * 4096
    r = np.random.default_rng(87)
    pos = r.uniform(-1, 1, (n, 3)).astype(np.float32)
    for c in range(n // 256):
        rot = (7 * c) & 15
        for k in range(8):
            a = c * 256 + rot + 32 * k
            pos[a + 16] = pos[a] + np.float32(1e-5) * np.array([1.0, 0.7, 0.3], np.float32)
    zero = np.zeros(n, np.float32)
    m = np.full(n, 1.0 / n, np.float32)
    arrs = (pos[:, 0].copy(), pos[:, 1].copy(), pos[:, 2].copy(), zero, zero, zero, m)
    out = {}
    for phases, buckets in ((5, 2), (1, 2), (5, 1), (3, 1)):
        g = gpu_sim(theta=0.5, eps=0.05, dt=0.01, build_phases=phases, build_buckets=buckets)
        g.load(*arrs)
        g.step(1)
        t = g.tree()
        ch = t["child"]
        front, seen = np.array([t["nnodes"]]), []
        while front.size:
            kids = ch[front - n].ravel()
            seen.append(kids[(kids >= 0) & (kids < n)])
            front = kids[kids >= n]
        seen = np.concatenate(seen)
        assert seen.size == n and np.unique(seen).size == n, (phases, buckets)
        st = g.stats()
        assert st["status"] == 0 and st["cells"] > n // 2, (phases, buckets, st["cells"])
        out[(phases, buckets)] = (t["sorted"], g.read())
        g.close()
    ref = out[(5, 2)]
    for key, (srt, state) in out.items():
        np.testing.assert_array_equal(srt, ref[0], err_msg=str(key))
        for k in KEYS:
            np.testing.assert_array_equal(state[k], ref[1][k], err_msg="%s %s" % (key, k))
