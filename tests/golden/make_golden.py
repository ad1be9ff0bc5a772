"""Generate the golden fixtures of tests/golden from the reference's own kernels.

Runs the reference project's six OpenCL kernels (kernels/nbody/*.cl), compiled as C++ by
oracle/build.py and driven by oracle/ref_emul.cpp with the reference host's launch
geometry (16 groups x 16 work-items), on seeded inputs, and stores inputs and per-step
outputs as .npz.  It needs the reference sources and therefore runs only where they are
mounted; the .npz files it writes are committed and travel with the tests.

The reference kernels fix THETA = 1.5 (theta^2), EPSILON = 0.0025 (eps^2) and
TIMESTEP = 0.025 at compile time (calculateforce.cl:14-18, integrate.cl:12), so every
fixture uses those constants.

Usage:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402

F32 = np.float32


def two_body():
    # universe/test/TwoBodyUniverse.java:8-18
    x = np.array([-1.1, 1.0], F32); y = np.array([-1.0, 1.1], F32); z = np.array([-1.0, 1.0], F32)
    m = np.array([1 / 8, 1 / 8], F32)
    return x, y, z, m


def eight_body():
    # universe/test/EightBodyUniverse.java:8-46
    p = [(-1.1, -1, -1), (1, -1, -1), (-1, 1, -1.1), (-1, -1, 1.1),
         (1, 1, -1), (-1, 1.1, 1), (1, -1, 1), (1, 1.1, 1)]
    x, y, z = (np.array([q[i] for q in p], F32) for i in range(3))
    return x, y, z, np.full(8, 1 / 8, F32)


def big_tree():
    # universe/test/BigTreeUniverse.java:8-25 (body 3 keeps mass 0, as in the generator)
    x = np.array([0, 1e-8, 10000, -10000], F32)
    y = np.array([0, 0, 10000, -10000], F32)
    z = np.array([0, 0, 10000, -10000], F32)
    m = np.array([0.1, 0.1, 0.1, 0.0], F32)
    return x, y, z, m


def random_cube(n, rng_range, seed):
    # RandomCubicUniverseGenerator.java:12-18: (u - 0.5) * range, masses 1/n
    rng = np.random.default_rng(seed)
    x, y, z = (((rng.random(n) - 0.5) * rng_range).astype(F32) for _ in range(3))
    return x, y, z, np.full(n, 1.0 / n, F32)


def uniform_ball(n, seed, vsigma=0.05):
    rng = np.random.default_rng(seed)
    pts = np.empty((0, 3))
    while pts.shape[0] < n:
        c = rng.random((2 * n, 3)) * 2 - 1
        pts = np.concatenate([pts, c[(c * c).sum(1) <= 1]])
    pts = pts[:n].astype(F32)
    v = (rng.standard_normal((n, 3)) * vsigma).astype(F32)
    return pts[:, 0].copy(), pts[:, 1].copy(), pts[:, 2].copy(), np.full(n, 1.0 / n, F32), v


CASES = {
    # name: (builder, steps)
    "two_body": (lambda: (*two_body(), None), 3),
    "eight_body": (lambda: (*eight_body(), None), 3),
    "big_tree": (lambda: (*big_tree(), None), 3),
    "cube_4096": (lambda: (*random_cube(4096, 6.0, 7), None), 3),
    "ball_16384": (lambda: uniform_ball(16384, 11), 2),
}


def make(name):
    build, steps = CASES[name]
    x, y, z, m, v = build()
    n = x.size
    if v is None:
        vx = vy = vz = np.zeros(n, F32)
    else:
        vx, vy, vz = (v[:, i].copy() for i in range(3))
    R = O.run_reference(x, y, z, vx, vy, vz, m, steps)
    if R["error"]:
        raise RuntimeError("reference reported error %d on %s" % (R["error"], name))
    out = dict(x0=x, y0=y, z0=z, vx0=vx, vy0=vy, vz0=vz, m=m,
               steps=np.int32(steps), theta2=F32(O.REFERENCE_THETA2), eps2=F32(O.REFERENCE_EPS2),
               dt=F32(O.REFERENCE_DT), maxdepth=np.int32(R["maxdepth"]),
               root_count=np.int32(R["root_count"]), sorted=R["sorted"], root=R["root"])
    for k in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az"):
        out[k] = R[k]
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print("%-12s n=%-6d steps=%d maxdepth=%d -> %s (%d bytes)" % (
        name, n, steps, R["maxdepth"], os.path.basename(path), os.path.getsize(path)))


if __name__ == "__main__":
    names = sys.argv[1:] or list(CASES)
    for nm in names:
        make(nm)
