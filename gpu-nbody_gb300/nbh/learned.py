"""Learned per-body opening angle: training data, training, installation, evaluation.

The model is an MLP 12 -> 64 -> 64 -> 1 that maps a body's features to log(theta).  Its
training data come from the method itself: on sampled bodies of a universe, force probes
at a grid of fixed angles give each body's relative force error against the FP64 direct
sum, and the target of a body is the largest angle whose error stays within `tau` (log
interpolation between grid angles).  Samples pair the features measured in the probe at
each grid angle with that target.  Training runs on the GPU (nbh_mlp_train: FP32 forward
and backward kernels, Adam) with a pinball loss at a low quantile, so that the predicted
angle errs on the safe side.  The fixed-angle walk stays the fallback and the yardstick of
the error: every evaluation measures the error against FP64.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib as L

GRID = (0.4, 0.5, 0.6, 0.7, 0.8, 0.9, 1.0)
HERE = os.path.dirname(os.path.abspath(__file__))
MODEL_DIR = os.path.join(HERE, "models")


def rel_error(ax, ay, az, rx, ry, rz):
    num = np.sqrt((ax - rx) ** 2 + (ay - ry) ** 2 + (az - rz) ** 2)
    den = np.sqrt(rx ** 2 + ry ** 2 + rz ** 2)
    return num / np.maximum(den, 1e-300)


def probe(sim, theta):
    """Force probe at the current positions with per-body theta (array) or fixed (None)."""
    n = sim.n
    out = [np.empty(n, np.float32) for _ in range(4)]
    inter = C.c_int64()
    th = None if theta is None else np.ascontiguousarray(theta, dtype=np.float32)
    sim._check(sim._L.nbh_force_probe(sim._h, None if th is None else th.ctypes.data,
                                      *[o.ctypes.data for o in out], C.byref(inter)))
    return out[0], out[1], out[2], out[3], inter.value


def features(sim, use_probe=True):
    f = np.empty((sim.n, L.NBH_MLP_FEATURES), np.float32)
    sim._check(sim._L.nbh_theta_features(sim._h, f.ctypes.data, int(use_probe)))
    return f


def theta_target(E, tau, grid=GRID, floor=0.3, monotone=True):
    """Largest angle with error <= tau per sample (columns of E, rows = grid angles), log-
    linearly interpolated between grid points; `floor` when even the smallest fails.
    monotone: the largest angle below which every grid angle meets tau (a body's error is
    not monotone in the angle -- cancellations make single angles pass by luck, and such
    a pass does not carry over to a walk with another angle); otherwise the largest
    passing grid angle."""
    lE = np.log(np.maximum(E, 1e-300))
    lt = np.log(np.asarray(grid))
    lt_tau = np.log(tau)
    out = np.full(E.shape[1], np.log(floor))
    for j in range(E.shape[1]):
        passing = lE[:, j] <= lt_tau
        if monotone:
            k = int(np.argmin(passing)) - 1 if not passing.all() else len(grid) - 1
            if k < 0:
                continue
        else:
            ok = np.where(passing)[0]
            if ok.size == 0:
                continue
            k = ok.max()
        if k == len(grid) - 1:
            out[j] = lt[-1]
            continue
        f = (lt_tau - lE[k, j]) / max(lE[k + 1, j] - lE[k, j], 1e-12)
        out[j] = lt[k] + np.clip(f, 0.0, 1.0) * (lt[k + 1] - lt[k])
    return out


def collect(sim, nsample, rng, grid=GRID):
    """Errors and features of nsample bodies at every grid angle (current positions).
    Returns (E [len(grid), S], F [len(grid), S, 12], interactions per grid angle)."""
    n = sim.n
    idx = np.sort(rng.choice(n, min(nsample, n), replace=False)).astype(np.int32)
    ref = sim.direct_f64(idx)
    E, F, I = [], [], []
    for th in grid:
        ax, ay, az, _, inter = probe(sim, np.full(n, th, np.float32))
        f = features(sim, use_probe=True)
        E.append(rel_error(ax[idx], ay[idx], az[idx], *ref))
        F.append(f[idx])
        I.append(inter)
    return np.stack(E), np.stack(F), np.array(I)


def init_params(seed=0):
    rng = np.random.default_rng(seed)
    W1 = rng.standard_normal((64, 12)) * np.sqrt(2.0 / 12)
    W2 = rng.standard_normal((64, 64)) * np.sqrt(2.0 / 64)
    W3 = rng.standard_normal(64) * np.sqrt(1.0 / 64)
    p = np.concatenate([W1.ravel(), np.zeros(64), W2.ravel(), np.zeros(64), W3, [np.log(0.6)]])
    return p.astype(np.float32)


def train(X, Y, quantile=0.2, iters=1500, lr=3e-3, seed=0, device=0, std_floor=0.05):
    """Normalise the features and fit the MLP on the device.  Returns the model dict."""
    X = np.asarray(X, dtype=np.float32)
    Y = np.asarray(Y, dtype=np.float32)
    mean = X.mean(0).astype(np.float32)
    std = np.maximum(X.std(0), std_floor).astype(np.float32)
    Xn = np.ascontiguousarray((X - mean) / std, dtype=np.float32)
    p = init_params(seed)
    loss = C.c_float()
    L.check(L.load().nbh_mlp_train(device, p.ctypes.data, Xn.ctypes.data, Y.ctypes.data, Xn.shape[0],
                                   float(quantile), int(iters), float(lr), C.byref(loss)))
    return {"params": p, "mean": mean, "inv_std": (1.0 / std).astype(np.float32), "loss": float(loss.value),
            "quantile": float(quantile)}


def set_grouping(sim, group_min):
    """1: each vote group walks with the smallest angle of its bodies; 0: per body."""
    sim._check(sim._L.nbh_set_theta_grouping(sim._h, int(bool(group_min))))


def install(sim, model, theta_min=0.3, theta_max=1.0, enable=True, every=None, group=None):
    """Switch the model on in `sim`; `every` = steps between evaluations, `group` = the
    grouping of nbh_set_theta_grouping (defaults: the model's own "every" and "group"
    entries, else 1 and 0)."""
    if every is None:
        every = int(model.get("every", 1))
    if group is None:
        group = int(model.get("group", 0))
    sim._check(sim._L.nbh_set_theta_interval(sim._h, int(every)))
    set_grouping(sim, group)
    p = np.ascontiguousarray(model["params"], dtype=np.float32)
    mu = np.ascontiguousarray(model["mean"], dtype=np.float32)
    inv = np.ascontiguousarray(model["inv_std"], dtype=np.float32)
    sim._check(sim._L.nbh_set_theta_model(sim._h, p.ctypes.data, p.size, mu.ctypes.data, inv.ctypes.data,
                                          float(model.get("theta_min", theta_min)),
                                          float(model.get("theta_max", theta_max)), int(bool(enable))))


def read_theta(sim):
    t = np.empty(sim.n, np.float32)
    sim._check(sim._L.nbh_read_theta(sim._h, t.ctypes.data))
    return t


def save(model, path):
    np.savez(path, **{k: np.asarray(v) for k, v in model.items()})


def load_model(path):
    d = np.load(path)
    return {k: (d[k] if d[k].ndim else d[k].item()) for k in d.files}


def default_model_path(name="theta_plummer"):
    return os.path.join(MODEL_DIR, name + ".npz")
