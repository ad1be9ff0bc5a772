"""Shared helpers of the test suite: GPU simulations through the C ABI and the oracle."""
from __future__ import annotations

import glob
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
GOLDEN_FILES = sorted(glob.glob(os.path.join(GOLDEN, "*.npz")))
KEYS = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az")


def gpu_sim(**kw):
    import nbh
    return nbh.Simulation(**kw)


def oracle_for(n, **kw):
    import oracle as O
    return O.Oracle(n, **kw)


def acc_rel(st, ref):
    a = np.stack([st["ax"], st["ay"], st["az"]]).astype(np.float64)
    r = np.stack([ref["ax"], ref["ay"], ref["az"]]).astype(np.float64)
    da = np.linalg.norm(a - r, axis=0)
    na = np.linalg.norm(r, axis=0)
    return da / np.maximum(na, 1e-30), da.max() / max(na.max(), 1e-30)


def plummer(n, seed=1):
    from nbh import universe as U
    return U.PlummerUniverseGenerator(seed=seed).arrays(n)


def ball(n, seed=1, vsigma=0.05):
    from nbh import universe as U
    return U.UniformBallUniverseGenerator(seed=seed, vsigma=vsigma).arrays(n)


def assert_same_tree(gt, ot, nbody, groot, oroot, gnbody_offset=0):
    """Walk the GPU tree (compact cell indexing) and the oracle tree (full indexing) from
    their roots in parallel: same child kinds, same bodies, same slot order."""
    stack = [(groot, oroot)]
    cells = 0
    while stack:
        gc, oc = stack.pop()
        cells += 1
        gch = gt["child"][gc - gt["nbody"]]
        och = ot["child"][oc]
        for k in range(8):
            g, o = int(gch[k]), int(och[k])
            if o < 0:
                assert g < 0, (gc, k)
            elif o < nbody:
                assert g == o + gnbody_offset, (gc, k, g, o)
            else:
                assert g >= gt["nbody"], (gc, k, g)
                stack.append((g, o))
    return cells
