"""The oracle (oracle/refbh.c) against the golden fixtures made by the reference's own
kernels (tests/golden/make_golden.py), and against the reference kernels live where
their sources are mounted.

Tolerances: the reference sums a cell's children in an order that depends on thread
timing (summarizetree.cl:84-150 adds children that were not ready later, last first), so
two runs of the reference itself differ by up to ~2e-7 of the acceleration scale; the
tree shape, the depth-first body order and the tree depth are exact.
"""
import glob
import os

import numpy as np
import pytest

import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FILES = sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))

ACC_REL_MAX = 5e-5      # per body |da| / |a|
ACC_REL_MEDIAN = 1e-6
ACC_SCALE_REL = 2e-6    # max |da| / max |a|
POS_SCALE_REL = 1e-6


def _oracle_for(G, **kw):
    n = G["x0"].size
    o = O.Oracle(n, theta2=float(G["theta2"]), eps2=float(G["eps2"]), dt=float(G["dt"]),
                 vote=16, fma=False, **kw)
    o.load(G["x0"], G["y0"], G["z0"], G["vx0"], G["vy0"], G["vz0"], G["m"])
    return o


def _check_step(st, G, s):
    a = np.stack([st["ax"], st["ay"], st["az"]])
    ar = np.stack([G["ax"][s], G["ay"][s], G["az"][s]])
    da = np.linalg.norm(a - ar, axis=0)
    na = np.linalg.norm(ar, axis=0)
    rel = da / np.maximum(na, 1e-30)
    assert rel.max() <= ACC_REL_MAX, rel.max()
    assert np.median(rel) <= ACC_REL_MEDIAN
    assert da.max() <= ACC_SCALE_REL * max(na.max(), 1e-30)
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        ref = G[k][s]
        scale = max(np.abs(ref).max(), 1e-30)
        assert np.abs(st[k] - ref).max() <= POS_SCALE_REL * scale, k


@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f)[:-4] for f in FILES])
def test_oracle_matches_reference_golden(path):
    G = np.load(path)
    o = _oracle_for(G)
    for s in range(int(G["steps"])):
        assert o.step() == 0
        _check_step(o.state(), G, s)
    t = o.tree_arrays()
    np.testing.assert_array_equal(t["sorted"], G["sorted"])
    assert o.maxdepth == int(G["maxdepth"])
    assert t["count"][o.nn] == int(G["root_count"]) == G["x0"].size


@pytest.mark.parametrize("name", ["two_body", "eight_body", "big_tree"])
def test_tiny_universes_bit_exact(name):
    """With at most one child cell per level nothing is summed out of order, so the
    restatement reproduces the reference bit for bit."""
    G = np.load(os.path.join(GOLDEN, name + ".npz"))
    o = _oracle_for(G)
    for s in range(int(G["steps"])):
        o.step()
        st = o.state()
        for k in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az"):
            np.testing.assert_array_equal(st[k], G[k][s], err_msg="%s step %d" % (k, s))


def test_reference_root_centre():
    """TestBoundingBox.testRoot (test/ch/fhnw/woipv/tests/TestBoundingBox.java:205-247):
    32768 bodies uniform in a cube of side 32768; root centre = 0.5*(min+max) within 1e-5."""
    n = 2048 * 16
    rng = np.random.default_rng(3)
    x, y, z = (((rng.random(n) - 0.5) * n).astype(np.float32) for _ in range(3))
    m = np.full(n, 1.0 / n, np.float32)
    o = O.Oracle(n)
    o.load(x, y, z, None, None, None, m)
    o.bbox()
    t = o.tree_arrays()
    for arr, c in ((x, t["x"]), (y, t["y"]), (z, t["z"])):
        root = np.float32(0.5) * (arr.min() + arr.max())
        assert abs(float(root) - float(c[o.nn])) < 1e-5


@pytest.mark.skipif(not O.reference_available(), reason="reference sources not mounted")
def test_oracle_matches_reference_live():
    """Fresh inputs through the reference kernels compiled here (not a stored fixture)."""
    n = 2048
    rng = np.random.default_rng(123)
    x, y, z = (((rng.random(n) - 0.5) * 4).astype(np.float32) for _ in range(3))
    v = (rng.standard_normal((3, n)) * 0.05).astype(np.float32)
    m = (rng.random(n) * 2 / n).astype(np.float32)
    R = O.run_reference(x, y, z, v[0], v[1], v[2], m, 2)
    assert R["error"] == 0
    G = dict(x0=x, y0=y, z0=z, vx0=v[0], vy0=v[1], vz0=v[2], m=m, theta2=O.REFERENCE_THETA2,
             eps2=O.REFERENCE_EPS2, dt=O.REFERENCE_DT, **{k: R[k] for k in
                                                          ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az")})
    o = _oracle_for(G)
    for s in range(2):
        o.step()
        _check_step(o.state(), G, s)
    np.testing.assert_array_equal(o.tree_arrays()["sorted"], R["sorted"])
    assert o.maxdepth == R["maxdepth"]
