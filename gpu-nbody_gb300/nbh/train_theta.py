"""Train the learned opening-angle model on the GPU and store it in nbh/models/.

  python gpu-nbody_gb300/nbh/train_theta.py [--n 1048576] [--out PATH]

  python gpu-nbody_gb300/nbh/train_theta.py --study     # ceiling of a per-body angle

Training data: uniform balls of 16,384 bodies and Plummer spheres (scale radius 1, mass 1)
of n bodies, two seeds each, each at its initial state and after 10 steps; per snapshot nbh.learned.collect() probes the
force at the angle grid on sampled bodies and measures the error against the FP64 direct
sum.  Candidate models are fitted for several error budgets tau (fractions of the fixed
theta = 0.5 p99 error) and loss quantiles, then validated on a third seed through the
production step path (features and BF16 inference inside the step, the model evaluated
every 8 steps), each with several floors of the predicted angle, on three held-out
spheres (16,384 sampled bodies each); of the candidates whose p99 error, averaged over one
evaluation cycle of steps and over the spheres, stays within 0.98 of the fixed-theta p99
over the same steps (and within 1.05 on every sphere), and whose worst step does not exceed
fixed theta's worst on average, the fastest is kept.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import nbh  # noqa: E402
from nbh import learned as LR  # noqa: E402
from nbh import universe as U  # noqa: E402


def evaluate(arrs, model, theta=0.5, eps=0.05, dt=0.01, nsample=16384, warm=3, cycle=None, timed=16, seed=17,
             device=0, every=None):
    """Fixed theta (plain) against the learned angle (if model) from the same initial
    state, through the production step: after `warm` steps, the relative force error
    against FP64 on `nsample` bodies at each of `cycle` consecutive steps (p99 mean and
    max over the steps, median), the mean interactions per step, and ms/step over
    `timed` further steps (host clock around synchronous steps).  `cycle` defaults to one
    whole evaluation cycle of the model (its interval, at least 8 steps), so that every
    phase of the cycle is measured once and both modes over the same step indices."""
    if cycle is None:
        k = every if every is not None else (int(model.get("every", 1)) if model is not None else 1)
        cycle = max(8, k)
    timed = max(timed, cycle) // cycle * cycle
    n = arrs[0].size
    idx = np.sort(np.random.default_rng(seed).choice(n, min(nsample, n), replace=False)).astype(np.int32)
    out = {}
    for mode in ("plain", "learned"):
        if mode == "learned" and model is None:
            continue
        with nbh.Simulation(theta=theta, eps=eps, dt=dt, device=device) as s:
            s.load(*arrs)
            if mode == "learned":
                LR.install(s, model, every=every)
            s.step(warm)
            p99, med, inter = [], [], []
            for _ in range(cycle):
                ref = s.direct_f64(idx)
                s.step(1)
                st = s.read()
                e = LR.rel_error(st["ax"][idx], st["ay"][idx], st["az"][idx], *ref)
                p99.append(float(np.percentile(e, 99)))
                med.append(float(np.median(e)))
                inter.append(int(s.stats()["interactions"]))
            s.step(2)
            t0 = time.perf_counter()
            s.step(timed)
            ms = 1e3 * (time.perf_counter() - t0) / timed
            out[mode] = {"p99": float(np.mean(p99)), "p99_max": float(np.max(p99)), "median": float(np.mean(med)),
                         "interactions": float(np.mean(inter)), "ms_per_step": ms}
            if mode == "learned":
                th = LR.read_theta(s)
                out[mode]["theta_mean"] = float(th.mean())
    return out


def study(n=1 << 20, seed=2024, grid=(0.4, 0.45, 0.5, 0.55, 0.6, 0.7, 0.8, 0.9, 1.0, 1.1, 1.2), fracs=(0.5, 0.7, 1.0),
          device=0, nsample=4096):
    """Ceiling of a per-body opening angle on a Plummer sphere: every body's relative force
    error at each fixed angle of `grid` (against a theta = 0.05 walk, itself checked against
    the FP64 direct sum on `nsample` bodies), then the walk with each body's own ideal angle
    (the largest grid angle, monotone, whose error stays within frac * p99 of theta = 0.5),
    whose interactions and p99 are compared with the fixed angles'.  Returns a dict."""
    arrs = U.PlummerUniverseGenerator(seed=seed).arrays(n)
    out = {"n": n, "fixed": {}, "ideal": {}}
    with nbh.Simulation(theta=0.5, eps=0.05, dt=0.01, device=device) as s:
        s.load(*arrs)
        s.step(3)
        idx = np.sort(np.random.default_rng(17).choice(n, min(nsample, n), replace=False)).astype(np.int32)
        f64 = s.direct_f64(idx)
        rx, ry, rz, _, ri = LR.probe(s, np.full(n, 0.05, np.float32))
        e_ref = LR.rel_error(rx[idx], ry[idx], rz[idx], *f64)
        out["reference_walk"] = {"theta": 0.05, "interactions": ri, "p99_vs_fp64": float(np.percentile(e_ref, 99))}
        E = []
        for th in grid:
            ax, ay, az, _, it = LR.probe(s, np.full(n, th, np.float32))
            e = LR.rel_error(ax, ay, az, rx, ry, rz)
            E.append(e)
            out["fixed"]["%.2f" % th] = {"interactions": it, "p50": float(np.median(e)), "p99": float(np.percentile(e, 99))}
        E = np.stack(E)
        p99 = out["fixed"]["0.50"]["p99"]
        for frac in fracs:
            T = np.exp(LR.theta_target(E, frac * p99, grid=tuple(grid), floor=0.3))
            ax, ay, az, _, it = LR.probe(s, T.astype(np.float32))
            e = LR.rel_error(ax, ay, az, rx, ry, rz)
            out["ideal"]["%.1f" % frac] = {"interactions": it, "p50": float(np.median(e)), "p99": float(np.percentile(e, 99)),
                                          "theta_mean": float(T.mean())}
    return out


FLOORS = (0.36, 0.4, 0.42, 0.45, 0.48)
EVERY = (8,)              # steps between evaluations of the model
TAU_FRACS = (0.55, 0.6, 0.65)
QUANTILES = (0.1,)
INIT_SEEDS = (0, 1, 2)    # initial weights of the network
VAL_SEEDS = (103, 104, 105)   # held-out Plummer spheres of the selection
# the p99 of one realisation moves by several per cent from sphere to sphere at the same
# settings: a candidate's p99 ratio, averaged over the held-out spheres, must stay within
# P99_MARGIN of fixed theta's, and on no single sphere above P99_WORST
P99_MARGIN = 0.98
P99_WORST = 1.05


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=1 << 20)
    ap.add_argument("--samples", type=int, default=6144)
    ap.add_argument("--out", default=LR.default_model_path())
    ap.add_argument("--previous", default=LR.default_model_path(),
                    help="a model that competes in the selection with its floor and interval re-searched")
    ap.add_argument("--iters", type=int, default=1500)
    ap.add_argument("--group", type=int, default=0, help="1: each vote group walks with its smallest angle")
    ap.add_argument("--study", action="store_true", help="measure the ceiling of a per-body angle and exit")
    args = ap.parse_args()
    if args.study:
        r = study(n=args.n)
        print(json.dumps(r, indent=1))
        fx = r["fixed"]
        for frac, v in r["ideal"].items():
            # the fixed angle with the same p99, by log-interpolating the fixed-angle curve
            ths = sorted(fx, key=float)
            p = [fx[t]["p99"] for t in ths]
            it = [fx[t]["interactions"] for t in ths]
            eq = float(np.interp(np.log(v["p99"]), np.log(p), np.log(it)))
            print("ideal per-body angle at tau = %s x p99(0.5): %.3e interactions, p99 %.2e; a fixed angle "
                  "with that p99: %.3e interactions (gain %.2fx)" % (frac, v["interactions"], v["p99"], np.exp(eq),
                                                                      np.exp(eq) / v["interactions"]))
        return
    t0 = time.time()
    rng = np.random.default_rng(1)
    Es, Fs = [], []
    # the two workloads the model is trained on: uniform balls of 16,384 bodies (dt 0.025)
    # and Plummer spheres of n bodies (dt 0.01), two seeds each, initial and after 10 steps
    sources = [("ball", seed, U.UniformBallUniverseGenerator(seed=seed, radius=1.0, vsigma=0.05).arrays(16384), 0.025)
               for seed in (201, 202)]
    sources += [("plummer", seed, U.PlummerUniverseGenerator(seed=seed).arrays(args.n), 0.01) for seed in (101, 102)]
    p99s = []
    for name, seed, arrs, dt in sources:
        with nbh.Simulation(theta=0.5, eps=0.05, dt=dt) as s:
            s.load(*arrs)
            for k in range(2):
                if k:
                    s.step(10)
                E, F, I = LR.collect(s, args.samples, rng)
                Es.append(E)
                Fs.append(F)
                if name == "plummer":
                    p99s.append(np.percentile(E[1], 99))
                print("snapshot %s seed %d part %d: p99 at theta 0.5 = %.3e, interactions %s"
                      % (name, seed, k, np.percentile(E[1], 99), I.tolist()), flush=True)
    p99_plain = float(np.median(p99s))
    vals = [U.PlummerUniverseGenerator(seed=sd).arrays(args.n) for sd in VAL_SEEDS]
    # fixed theta over the same steps as each candidate: one evaluation cycle of its interval
    base = {(v, k): evaluate(val, None, cycle=max(8, k))["plain"] for v, val in enumerate(vals) for k in EVERY}
    print("validation plain:", {str(k): b for k, b in base.items()}, flush=True)
    best = None

    def consider(model, floor, every, info):
        nonlocal best
        model = dict(model)
        model["theta_min"] = floor
        model["every"] = every
        rs = []
        for v, val in enumerate(vals):
            r = evaluate(val, model)["learned"]
            b = base[(v, every)]
            r.update({"speedup": b["ms_per_step"] / r["ms_per_step"], "p99_ratio": r["p99"] / b["p99"],
                      "p99_max_ratio": r["p99_max"] / b["p99_max"],
                      "interaction_gain": b["interactions"] / r["interactions"]})
            rs.append(r)
        r = dict(info, theta_min=floor, every=every, loss=float(model.get("loss", 0.0)),
                 speedup=float(np.mean([x["speedup"] for x in rs])),
                 interaction_gain=float(np.mean([x["interaction_gain"] for x in rs])),
                 p99_ratio=float(np.mean([x["p99_ratio"] for x in rs])),
                 p99_ratio_worst=max(x["p99_ratio"] for x in rs),
                 p99_max_ratio=float(np.mean([x["p99_max_ratio"] for x in rs])),
                 ms_per_step=float(np.mean([x["ms_per_step"] for x in rs])), per_seed=rs)
        print(json.dumps({k: v for k, v in r.items() if k != "per_seed"}), flush=True)
        if (r["p99_ratio"] <= P99_MARGIN and r["p99_max_ratio"] <= 1.0 and r["p99_ratio_worst"] <= P99_WORST
                and (best is None or r["speedup"] > best[1]["speedup"])):
            best = (model, r)

    # the model in place (if any) competes with its inference-time settings re-searched
    if os.path.exists(args.previous):
        prev = LR.load_model(args.previous)
        prev.pop("validation", None)
        for floor, every in [(f, e) for f in FLOORS for e in EVERY]:
            consider(prev, floor, every, {"source": "previous model"})
    X = np.concatenate([F.reshape(-1, 12) for F in Fs])
    for tau_frac in TAU_FRACS:
        Y = np.concatenate([np.tile(LR.theta_target(E, tau_frac * p99_plain), E.shape[0]) for E in Es])
        for q, init in [(q, i) for q in QUANTILES for i in INIT_SEEDS]:
            model = LR.train(X, Y, quantile=q, iters=args.iters, seed=init)
            model.update({"theta_max": 1.0, "tau_frac": tau_frac, "tau": tau_frac * p99_plain,
                          "group": args.group, "init_seed": init})
            # the angle's floor is an inference-time clamp: a floor too low lets a few groups
            # walk at a very small angle, and their long walks become the launch's tail
            for floor, every in [(f, e) for f in FLOORS for e in EVERY]:
                consider(model, floor, every, {"source": "trained", "tau_frac": tau_frac, "quantile": q,
                                               "init_seed": init})
    if best is None:
        raise SystemExit("no candidate met the fixed-theta p99 error")
    model, r = best
    model["validation"] = json.dumps({"plain": {str(k): b for k, b in base.items()}, "learned": r})
    os.makedirs(os.path.dirname(args.out), exist_ok=True)
    LR.save(model, args.out)
    print("saved %s: %.3fx speed, %.3fx fewer interactions at p99 ratio %.3f (%.0f s)"
          % (args.out, r["speedup"], r["interaction_gain"], r["p99_ratio"], time.time() - t0))


if __name__ == "__main__":
    main()
