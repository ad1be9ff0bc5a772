"""CPU references of the learned opening-angle network (test infrastructure only).

* forward/grad: the 12 -> 64 -> 64 -> 1 ReLU MLP and its pinball-loss gradient in FP64,
  against which the device's FP32 training kernels are checked;
* forward_bf16: the same network with inputs, weights and hidden activations rounded to
  BF16 (round to nearest even) and FP32 sums, the arithmetic of the tensor-core inference;
* features_from_tree: the 12 per-body features recomputed from a tree read back with
  nbh_read_tree and a force probe's outputs.
"""
from __future__ import annotations

import numpy as np

NIN, NHID = 12, 64
NPARAMS = NHID * NIN + NHID + NHID * NHID + NHID + NHID + 1


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + NHID * NIN].reshape(NHID, NIN); o += NHID * NIN
    b1 = p[o:o + NHID]; o += NHID
    W2 = p[o:o + NHID * NHID].reshape(NHID, NHID); o += NHID * NHID
    b2 = p[o:o + NHID]; o += NHID
    W3 = p[o:o + NHID]; o += NHID
    b3 = p[o]
    return W1, b1, W2, b2, W3, b3


def forward(p, X):
    W1, b1, W2, b2, W3, b3 = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    h1 = np.maximum(X @ W1.T + b1, 0.0)
    h2 = np.maximum(h1 @ W2.T + b2, 0.0)
    return h2 @ W3 + b3


def grad(p, X, T, q):
    """Mean pinball loss of quantile q and its gradient w.r.t. the parameters (FP64).
    At a zero residual the derivative of the residual's negative side is used."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    X = np.asarray(X, dtype=np.float64)
    T = np.asarray(T, dtype=np.float64)
    n = X.shape[0]
    h1 = np.maximum(X @ W1.T + b1, 0.0)
    h2 = np.maximum(h1 @ W2.T + b2, 0.0)
    y = h2 @ W3 + b3
    r = T - y
    loss = np.where(r > 0, q * r, (q - 1.0) * r).mean()
    dy = np.where(r > 0, -q, 1.0 - q) / n
    dW3 = h2.T @ dy
    db3 = dy.sum()
    dh2 = np.outer(dy, W3) * (h2 > 0)
    dW2 = dh2.T @ h1
    db2 = dh2.sum(0)
    dh1 = (dh2 @ W2) * (h1 > 0)
    dW1 = dh1.T @ X
    db1 = dh1.sum(0)
    g = np.concatenate([dW1.ravel(), db1, dW2.ravel(), db2, dW3, [db3]])
    return loss, g


def bf16(x):
    """Round float32 values to BF16 (nearest even), returned as float32."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def forward_bf16(p, Xn):
    W1, b1, W2, b2, W3, b3 = (np.asarray(a, dtype=np.float32) for a in unpack(p))
    x = bf16(np.asarray(Xn, dtype=np.float32))
    h1 = np.maximum(x @ bf16(W1).T + b1, 0.0).astype(np.float32)
    h2 = np.maximum(bf16(h1) @ bf16(W2).T + b2, 0.0).astype(np.float32)
    return (bf16(h2) @ bf16(W3) + np.float32(b3)).astype(np.float32)


def features_from_tree(tree, x, y, z, probe_acc, ebound, theta_prev, eps):
    """Features of every body of a single-universe sim from its tree arrays
    (Simulation.tree()), positions and the previous walk's outputs."""
    n = tree["nbody"]
    nn = tree["nnodes"]
    child = tree["child"]
    node4 = tree["node4"].astype(np.float64)
    count = tree["count"]
    bottom = tree["bottom"]
    parent = np.full(nn + 1, -1, np.int64)
    level = np.zeros(nn + 1, np.int64)
    for c in range(nn, bottom - 1, -1):          # parents before children
        for ch in child[c - n]:
            if ch >= 0:
                parent[ch] = c
                if ch >= n:
                    level[ch] = level[c] + 1
    R = float(tree["radius"][0])
    com = node4[nn, :3]
    M = node4[nn, 3]
    pos = np.stack([x, y, z], 1).astype(np.float64)
    leaf = parent[:n]
    up = np.where(parent[leaf] >= 0, parent[leaf], leaf)
    lv = level[leaf]
    h = R * np.ldexp(1.0, -lv)
    nl = count[leaf - n].astype(np.float64)
    nu = count[up - n].astype(np.float64)
    ml = node4[leaf, 3]
    d = np.sqrt(((pos - com) ** 2).sum(1)) + 1e-12
    a = np.asarray(probe_acc, dtype=np.float64)
    am = np.sqrt((a ** 2).sum(1)) + 1e-30
    eb = np.maximum(np.asarray(ebound, dtype=np.float64), 0.0)
    return np.stack([
        np.log10(am), np.log10(eb / am + 1e-30), np.log10(np.maximum(theta_prev, 1e-6)),
        np.log10(d / R + 1e-12), np.log10(nl + 1.0), lv * 0.05, np.log10(nu + 1.0),
        np.log10(nl / h ** 3 + 1e-30), np.log10(np.maximum(ml, 0.0) / M + 1e-30),
        np.log10(am * d * d / M + 1e-30), np.log10(eps / h), np.log10(h / d)], 1)
