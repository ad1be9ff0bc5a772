#!/usr/bin/env python
"""Benchmark of the Barnes-Hut step: ms/step on a 1,048,576-body Plummer sphere.

Workload (seeded synthetic input of the named shape; no dataset is involved): Plummer
sphere, scale radius 1, total mass 1, equal masses, velocities from the distribution
function; theta 0.5, eps 0.05, dt 0.01, G 1.  A step is one full pass of the pipeline
bounding box -> octree build -> summarize -> sort -> force -> integrate over the whole
universe (one CUDA graph launch).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl nbh|reference]

value  = device time per step (CUDA events on the sim's stream, L2 flushed by a 256 MiB
         write before every timed step, inputs resident in HBM), max over ranks.
e2e    = the same step through the C ABI with host arrays: each step writes the state
         (x, y, z, v, a) from pinned host memory, steps, and reads it back, in one
         nbh_step_io call (the three separate calls are timed beside it).
Under torchrun every rank runs an independent replica (the step does not shard).
The reference arm (--impl reference) times the oracle port of the reference kernels
(oracle/refbh.c, OpenMP over all host cores) on the same workload; the reference's
OpenCL kernels cannot run on these machines (no JVM, no OpenCL 2.0 CPU runtime).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "gpu-nbody_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "ms/step at 1M bodies, plain vs learned-theta at equal p99 force error; Gint/s"
DEFAULT_VOTE = 64                   # libnbh's default vote width (nbh_config_default)


def graph_launches(build_phases=5, build_buckets=1):
    """Kernels in one fixed-angle step graph: bbox, the build's launches, link, summarize,
    sort, force, the work-item order of the next force launch, integrate.  The build is
    `build_phases` lock phases, or with the bucketed completion: five phases -> the three
    lock phases of the 1/16 sample and one bucketed pass (locate, alloc, scatter, subtree
    build); three phases -> one lock phase (1/256) and two bucketed passes."""
    if build_phases == 1 or build_buckets == 2:
        build = build_phases
    elif build_phases == 5:
        build = 3 + 4
    else:
        build = 1 + 2 * 4
    return 7 + build
FLOPS_PER_INTERACTION = 20          # 3 sub, 3 fma (d^2+eps^2), rsqrt, 3 mul, 3 fma, ~7 more
HBM_FALLBACK_GBS = 6800.0
# DRAM bytes (read + write) of one force launch (vote width 64) on the 1,048,576-body
# Plummer workload, from one full ncu capture of that launch (dram__bytes_read.sum +
# dram__bytes_write.sum).
FORCE_TRAFFIC_BYTES_1M = 222_678_016 + 25_789_440

# Algorithmic bytes per body / per cell of the memory-bound stages (minimum traffic:
# every byte read and written once).
STAGE_BYTES = {
    "bbox": lambda n, c: 16 * n,                       # float4 node reads
    "build": lambda n, c: 16 * n + 4 * n + 52 * c,     # body read, parent write, cell init
    "summarize": lambda n, c: 20 * n + 80 * c,         # child nodes read, COM/count/slots written
    "sort": lambda n, c: 40 * c + 4 * n,               # slots + counts + starts, sorted written
    "integrate": lambda n, c: 80 * n,                  # node4, vel, acc read; node4, vel written
}


def _env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", HBM_FALLBACK_GBS)), "measured (MEASURED_PEAKS.json)"
    return HBM_FALLBACK_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


# Workloads (seeded synthetic inputs of the shapes the benchmark cases name).  "plummer"
# is the headline; the others are the remaining cases of the same step, measured with
# the same protocol.
WORKLOADS = {
    "plummer": {"n": 1 << 20, "dt": 0.01, "precise": False,
                "what": "Plummer sphere a=1 M=1, equal masses, DF velocities"},
    # 16K bodies make only 256 groups of 64: the tuner may pick a narrower vote (more groups)
    "ball": {"n": 16384, "dt": 0.025, "precise": False, "tune_vote": True,
             "what": "uniform unit ball, equal masses 1/N, Gaussian velocities sigma 0.05"},
    "disc": {"n": 1 << 22, "dt": 0.01, "precise": True,
             "what": "exponential disc rd=1 zd=0.1 (near-circular velocities) + central mass 0.1 "
                     "+ 10% Plummer halo; Kahan-compensated updates, FP64 extent/root COM"},
    "ensemble": {"n": 256, "dt": 0.01, "precise": False,
                 "what": "256 independent Plummer spheres, N per universe log-uniform in "
                         "[1024, 65536], all advanced in one graph per step"},
}


def ensemble_counts(nuniv, seed, lo=1024, hi=65536):
    import numpy as np
    r = np.random.default_rng(seed)
    return np.exp(r.uniform(np.log(lo), np.log(hi), nuniv)).astype(np.int64).astype(np.int32)


def workload(args, seed):
    """(arrays x y z vx vy vz m, per-universe counts or None)."""
    import numpy as np
    from nbh import universe as U
    if args.workload == "plummer":
        return U.PlummerUniverseGenerator(seed=seed, a=1.0, M=1.0).arrays(args.n), None
    if args.workload == "ball":
        return U.UniformBallUniverseGenerator(seed=seed, radius=1.0, vsigma=0.05).arrays(args.n), None
    if args.workload == "disc":
        return U.DiscGalaxyGenerator(seed=seed, rd=1.0, zd=0.1, center_mass=0.1,
                                     halo_frac=0.1).arrays(args.n), None
    counts = ensemble_counts(args.n, seed)
    parts = [U.PlummerUniverseGenerator(seed=seed * 1000 + u, a=1.0, M=1.0).arrays(int(c))
             for u, c in enumerate(counts)]
    return tuple(np.concatenate([p[k] for p in parts]) for k in range(7)), counts


def shard_universes(counts, world, rank):
    """Universes of a batch for one rank: greedy balancing of sum N log N (largest first,
    each to the least loaded rank; deterministic).  Ranks share no data, so the batch
    shards without a collective on the data path."""
    import numpy as np
    counts = np.asarray(counts, dtype=np.int64)
    cost = counts * np.log2(np.maximum(counts, 2))
    order = np.argsort(-cost, kind="stable")
    load = np.zeros(world)
    owner = np.empty(counts.size, np.int64)
    for u in order:
        r = int(np.argmin(load))
        owner[u] = r
        load[r] += cost[u]
    return np.flatnonzero(owner == rank)


def select_universes(arrs, counts, keep):
    """The arrays and counts of the universes `keep` (indices, ascending) of a batch."""
    import numpy as np
    offs = np.concatenate([[0], np.cumsum(counts)])
    idx = np.concatenate([np.arange(offs[u], offs[u + 1]) for u in keep])
    return tuple(a[idx] for a in arrs), np.asarray(counts)[keep]


def reduce_sum(x, dist=None, device="cpu"):
    """Sum of x over the ranks of the default process group (x itself without one)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def reduce_max(x, dist=None, device="cpu"):
    """Maximum of x over the ranks of the default process group (x itself without one)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _oracles(arrs, counts, args):
    """One oracle port instance per universe (the port holds a single universe)."""
    import oracle as O
    bounds = [0, arrs[0].size] if counts is None else [0] + list(__import__("numpy").cumsum(counts))
    out = []
    for a, b in zip(bounds[:-1], bounds[1:]):
        o = O.Oracle(int(b - a), theta=args.theta, eps=args.eps, dt=args.dt, vote=args.vote_width, fma=True)
        o.load(*[v[a:b] for v in arrs])
        out.append(o)
    return out


def cpu_step_time(arrs, counts, args, max_seconds=25.0):
    """Oracle port (OpenMP, all host threads) on the same workload: seconds per step."""
    os_ = _oracles(arrs, counts, args)
    t0 = time.perf_counter()
    for o in os_:
        o.step()                               # warm-up (page faults, thread start)
    first = time.perf_counter() - t0
    steps = max(1, min(3, int(max_seconds / max(first, 1e-3))))
    t0 = time.perf_counter()
    for o in os_:
        o.step(steps)
    return (time.perf_counter() - t0) / steps, steps, sum(o.interactions for o in os_)


def run_reference(args):
    rank = _env_int("RANK", 0)
    if rank != 0:
        return 0
    arrs, counts = workload(args, args.seed)
    args.vote_width = args.vote or DEFAULT_VOTE
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    os_ = _oracles(arrs, counts, args)
    for _ in range(args.warmup):
        for o in os_:
            o.step()
    t = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        for o in os_:
            o.step()
        t.append(time.perf_counter() - t0)
    ms = 1e3 * sum(t) / len(t)
    nb = arrs[0].size
    line = {
        "impl": "reference", "metric": METRIC, "value": ms, "unit": "ms/step", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": _config(args, nb, counts),
        "cpu_baseline": {"value": ms, "unit": "ms/step", "cores": cores, "kind": "port",
                         "sample": "%d full steps of the %d-body %s workload (oracle/refbh.c, "
                                   "OpenMP force pass)" % (args.steps, nb, args.workload)},
        "e2e": {"value": ms, "unit": "ms/step", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gint_per_s": sum(o.interactions for o in os_) / (ms * 1e-3) / 1e9,
        "note": "the reference's OpenCL kernels need an OpenCL 2.0 runtime and a JVM, absent on "
                "this box; its CPU restatement (oracle/refbh.c) is timed instead",
    }
    print(json.dumps(line))
    return 0


def _config(args, nbodies=None, counts=None):
    w = WORKLOADS[args.workload]
    c = {"workload": "%s-%d" % (args.workload, args.n), "n_bodies": nbodies or args.n,
         "distribution": w["what"], "theta": args.theta, "eps": args.eps, "dt": args.dt, "G": 1.0,
         "vote_width": args.vote_width, "precise": w["precise"],
         "l2": "flushed before every timed step (256 MiB write)", "parallelism": "replicas",
         "error_samples": getattr(args, "error_samples", None)}
    if counts is not None:
        c.update({"universes": len(counts), "min_universe": int(min(counts)), "max_universe": int(max(counts))})
    if getattr(args, "force_list", 0):
        c["force_walk"] = "list" if args.force_list == 1 else "per-visit"
    return c


def _cycle_error(sim, idx, steps, O, np):
    """Relative force error against the FP64 direct sum over `steps` consecutive steps: at
    each step, the accelerations of the sampled bodies `idx` against the direct sum at the
    positions that step starts from.  With `steps` = the learned model's evaluation
    interval every phase of its cycle is measured once.  p99 and median per step, their
    mean and the worst step's p99, and the mean interactions per step."""
    p99, med, inter, errs = [], [], [], []
    for _ in range(steps):
        ref = sim.direct_f64(idx)
        sim.step(1)
        st = sim.read()
        e = O.rel_force_error(st["ax"][idx], st["ay"][idx], st["az"][idx], *ref)
        errs.append(e)
        p99.append(float(np.percentile(e, 99)))
        med.append(float(np.median(e)))
        inter.append(int(sim.stats()["interactions"]))
    return {"p99": float(np.mean(p99)), "p99_max": float(np.max(p99)), "median": float(np.mean(med)),
            "p99_per_step": p99, "steps": steps, "samples": int(idx.size), "vs": "FP64 direct sum",
            "interactions": float(np.mean(inter)), "_errors": np.stack(errs)}


def _p99_ratio_interval(el, ep, np, reps=200, seed=5):
    """Paired bootstrap over the sampled bodies (the same bodies in both arms, every step):
    the 2.5 and 97.5 percentiles of mean-over-steps p99(learned) / p99(plain)."""
    rng = np.random.default_rng(seed)
    n = el.shape[1]
    r = []
    for _ in range(reps):
        b = rng.integers(0, n, n)
        r.append(np.percentile(el[:, b], 99, axis=1).mean() / np.percentile(ep[:, b], 99, axis=1).mean())
    return [float(np.percentile(r, 2.5)), float(np.percentile(r, 97.5))]


def _stage_cycle(sim, steps, flush_l2, stream, torch):
    """Per-stage device times of `steps` consecutive stage-timed steps (L2 flushed before
    each): the mean of each stage and, per step, the force and learned-angle stages."""
    keys = ("ms_bbox", "ms_build", "ms_summarize", "ms_sort", "ms_theta", "ms_force", "ms_integrate", "ms_step")
    acc = {k: 0.0 for k in keys}
    force, theta = [], []
    for _ in range(steps):
        flush_l2(stream)
        sim.step(1)
        s2 = sim.stats()
        for k in keys:
            acc[k] += s2[k] / steps
        force.append(s2["ms_force"])
        theta.append(s2["ms_theta"])
    return acc, force, theta, sim.stats()


def _timed_steps(sim, steps, flush_l2, stream, torch, dev):
    """Device time of `steps` single-step graph launches, L2 flushed before each."""
    torch.cuda.synchronize(dev)
    evs = []
    for _ in range(steps):
        flush_l2(stream)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.step_async(1)
        e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize(dev)
    st = sim.stats()
    if st["status"] != 0:
        raise RuntimeError("device status %d during the timed steps" % st["status"])
    return [a.elapsed_time(b) for a, b in evs], st


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="nbh", choices=["nbh", "reference"])
    ap.add_argument("--workload", default="plummer", choices=sorted(WORKLOADS))
    ap.add_argument("--n", type=int, default=None,
                    help="bodies (universes for the ensemble); default per workload")
    ap.add_argument("--vote", type=int, default=None, help="vote width (16, 32, 64; default: the library's)")
    ap.add_argument("--theta", type=float, default=0.5)
    ap.add_argument("--eps", type=float, default=0.05)
    ap.add_argument("--dt", type=float, default=None)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch geometry")
    ap.add_argument("--tune-vote", action="store_true",
                    help="let the autotuner pick the vote width too (changes the interaction set)")
    ap.add_argument("--error-samples", type=int, default=16384,
                    help="bodies sampled for the FP64 error (the same bodies in both arms, every step)")
    ap.add_argument("--profile-only", action="store_true",
                    help="load, warm up and run the timed steps only (for ncu captures)")
    ap.add_argument("--profile-learned", action="store_true",
                    help="a --profile-only run steps with the learned per-body angle")
    ap.add_argument("--force-threads", type=int, default=0,
                    help="force launch geometry of a --profile-only run (0: the library default)")
    ap.add_argument("--stack-cap", type=int, default=0,
                    help="stack entries per vote group of a --profile-only run (0: the library default)")
    ap.add_argument("--force-list", type=int, default=0, choices=(0, 1, 2),
                    help="nbh_config.force_list: 1 the list walk, 2 the per-visit walk, 0 the library "
                         "default (the list walk except in precise mode)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    w = WORKLOADS[args.workload]
    args.tune_vote = args.tune_vote or bool(w.get("tune_vote"))
    if args.n is None:
        args.n = w["n"]
    if args.dt is None:
        args.dt = w["dt"]

    if args.impl == "reference":
        return run_reference(args)

    import numpy as np
    import torch

    import nbh
    import oracle as O
    from nbh import learned as LR

    rank, world, local = _env_int("RANK", 0), _env_int("WORLD_SIZE", 1), _env_int("LOCAL_RANK", 0)
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    if args.workload == "ensemble":
        # one ensemble for the whole job, its universes sharded across the ranks
        arrs, counts = workload(args, args.seed)
        if world > 1:
            arrs, counts = select_universes(arrs, counts, shard_universes(counts, world, rank))
    else:
        arrs, counts = workload(args, args.seed + rank)     # an independent replica per rank
    n = arrs[0].size
    precise = WORKLOADS[args.workload]["precise"]

    def new_sim(**kw):
        s_ = nbh.Simulation(theta=args.theta, eps=args.eps, dt=args.dt, device=local, precise=precise,
                            vote_width=args.vote, force_list=args.force_list, **kw)
        if counts is None:
            s_.load(*arrs)
        else:
            s_.load_batch(counts, *arrs)
        return s_
    idx = np.sort(np.random.default_rng(17).choice(n, min(args.error_samples, n), replace=False)).astype(np.int32)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def flush_l2(stream):
        with torch.cuda.stream(stream):
            flush.zero_()

    def max_over_ranks(x):
        return reduce_max(x, dist, dev)

    # ---- plain fixed theta: warm-up, error of one step, timed steps ---------------------
    sim = new_sim(**({"force_threads": args.force_threads, "stack_cap": args.stack_cap} if args.profile_only else {}))
    args.vote_width = int(sim.config.vote_width)
    model_path = LR.default_model_path()
    model = LR.load_model(model_path) if (not args.no_learned and os.path.exists(model_path)) else None
    if args.profile_only and args.profile_learned and model is not None:
        LR.install(sim, model)
    stream = torch.cuda.ExternalStream(sim.stream, device=dev)
    for _ in range(args.warmup):
        flush_l2(stream)
        sim.step(1)
    # launch geometry picked by the library's autotuner (changes no result); profile runs
    # keep the default geometry so that their launch lists hold only the step's kernels
    tune = None if (args.no_autotune or args.profile_only) else sim.autotune(vote=args.tune_vote)
    if tune is not None:
        args.vote_width = int(tune["vote_width"])
    # the error of both arms over the same steps: one full evaluation cycle of the learned
    # model (every phase of it once), from the same step index
    cycle = max(8, int(model.get("every", 1))) if model is not None else 8
    force_error = None if args.profile_only else _cycle_error(sim, idx, cycle, O, np)
    clocks = ClockSampler(local) if rank == 0 else None
    if clocks:
        clocks.start()
    if dist:
        dist.barrier()
    step_ms, st = _timed_steps(sim, args.steps, flush_l2, stream, torch, dev)
    if dist:
        dist.barrier()
    clock_info = clocks.stop() if clocks else None
    ms = max_over_ranks(sum(step_ms) / len(step_ms))
    interactions = int(st["interactions"])
    if args.profile_only:
        if rank == 0:
            print(json.dumps({"profile_only": True, "ms_per_step": ms, "interactions": interactions}))
        sim.close()
        return 0

    # per-stage device times (eager launches with events between stages)
    hbm_peak, peak_src = _peaks()
    geometry = {} if tune is None else {"force_threads": tune["force_threads"], "stack_cap": tune["stack_cap"],
                                        "build_phases": tune["build_phases"], "build_buckets": tune["build_buckets"],
                                        "top_phase": tune["top_phase"]}
    if tune is not None and args.tune_vote:
        args.vote = int(tune["vote_width"])      # the other sims walk with the chosen width too
    ts = new_sim(stage_timing=True, **geometry)
    ts.step(2)
    tstream = torch.cuda.ExternalStream(ts.stream, device=dev)
    acc, _, _, s2 = _stage_cycle(ts, 5, flush_l2, tstream, torch)
    acc.pop("ms_theta")
    cells = int(s2["cells"])
    inter_ts = int(s2["interactions"])
    ts.close()
    stages = {}
    for name in ("bbox", "build", "summarize", "sort", "integrate"):
        t_ms = acc["ms_" + name]
        b = STAGE_BYTES[name](n, cells)
        gbs = b / (t_ms * 1e-3) / 1e9 if t_ms > 0 else None
        stages[name] = {"ms": t_ms, "algorithmic_bytes": b, "GB_per_s": gbs,
                        "frac_of_hbm": (gbs / hbm_peak) if gbs else None}
    force_ms = acc["ms_force"]
    stages["force"] = {"ms": force_ms, "interactions": inter_ts}
    fp32 = __import__("ctypes").c_double()
    nbh._lib.check(nbh._lib.load().nbh_measure_fp32_peak(local, __import__("ctypes").byref(fp32)))
    achieved = FLOPS_PER_INTERACTION * inter_ts / (force_ms * 1e-3) / 1e12
    kname = "force_kernel64" if args.vote_width == 64 else "force_kernel<%d,FMA>" % args.vote_width
    roofline = {"bound": "fp32", "kernel": kname, "achieved": achieved,
                "peak": fp32.value, "unit": "TFLOP/s", "frac": achieved / fp32.value,
                "traffic": FORCE_TRAFFIC_BYTES_1M if (args.workload == "plummer" and n == 1 << 20
                                                      and args.vote_width == DEFAULT_VOTE) else None,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one force "
                                  "launch of this workload (full capture)",
                "flops_per_interaction": FLOPS_PER_INTERACTION,
                "peak_source": "measured FP32 FMA loop on this GPU (nbh_measure_fp32_peak); "
                               "MEASURED_PEAKS.json holds only HBM and bf16 peaks",
                "hbm_peak_GBps": hbm_peak, "hbm_peak_source": peak_src}

    # end to end through the C ABI with pinned host buffers
    keys = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az")
    hin = {k: torch.empty(n, dtype=torch.float32, pin_memory=True).numpy() for k in keys}
    hout = {k: torch.empty(n, dtype=torch.float32, pin_memory=True).numpy() for k in keys}
    cur = sim.read()
    for k in keys:
        hin[k][:] = cur[k]
    e2e_steps = max(3, min(args.steps, 10))
    torch.cuda.synchronize(dev)
    # nbh_step_io: the state written from the pinned arrays, one step, the state read back,
    # one wait at the end
    e2e_ev = []
    t_wall = time.perf_counter()
    for _ in range(e2e_steps):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ev[0].record(stream)
        sim.step_io(1, write=hin, read=hout)
        ev[1].record(stream)
        e2e_ev.append(ev)
    torch.cuda.synchronize(dev)
    wall_ms = 1e3 * (time.perf_counter() - t_wall) / e2e_steps
    e2e_ms = sum(ev[0].elapsed_time(ev[1]) for ev in e2e_ev) / e2e_steps
    # the same through the three calls nbh_write, nbh_step, nbh_read (each waits); device
    # time of each part, the gaps between the calls included
    three = []
    for _ in range(e2e_steps):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        ev[0].record(stream)
        sim.write(*[hin[k] for k in keys])
        ev[1].record(stream)
        sim.step(1)
        ev[2].record(stream)
        sim.read_into(*[hout[k] for k in keys])
        ev[3].record(stream)
        three.append(ev)
    torch.cuda.synchronize(dev)
    e2e_three = {"ms": sum(ev[0].elapsed_time(ev[3]) for ev in three) / e2e_steps}
    e2e_three.update({name: sum(ev[i].elapsed_time(ev[i + 1]) for ev in three) / e2e_steps
                      for i, name in enumerate(("write_ms", "step_ms", "read_ms"))})
    if dist:
        t = torch.tensor([e2e_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())

    # ---- learned per-body theta: same protocol ----------------------------------------
    learned = None
    if model is not None:
        ls = new_sim(**geometry)
        LR.install(ls, model)
        lstream = torch.cuda.ExternalStream(ls.stream, device=dev)
        for _ in range(args.warmup):
            flush_l2(lstream)
            ls.step(1)
        # the same step indices as the plain arm's error, the same sampled bodies
        lerr = _cycle_error(ls, idx, cycle, O, np)
        # timed steps: a whole number of model cycles, so every phase weighs the same
        lsteps = max(cycle, (args.steps + cycle - 1) // cycle * cycle)
        lstep_ms, lst = _timed_steps(ls, lsteps, flush_l2, lstream, torch, dev)
        lms = max_over_ranks(sum(lstep_ms) / len(lstep_ms))
        th = LR.read_theta(ls)
        ls.close()
        # the learned step's own stages over one cycle: features + inference (theta), the
        # walks with and without the error-bound recording
        lt = new_sim(stage_timing=True, **geometry)
        LR.install(lt, model)
        lt.step(args.warmup)
        ltstream = torch.cuda.ExternalStream(lt.stream, device=dev)
        lacc, lforce, ltheta, _ = _stage_cycle(lt, cycle, flush_l2, ltstream, torch)
        lt.close()
        learned = {
            "ms_per_step": lms / (world if args.workload != "ensemble" else 1), "speedup_vs_plain": ms / lms,
            "timed_steps": lsteps,
            "force_error": lerr, "p99_vs_plain": lerr["p99"] / force_error["p99"],
            "p99_max_vs_plain": lerr["p99_max"] / force_error["p99_max"],
            "p99_vs_plain_95ci": _p99_ratio_interval(lerr.pop("_errors"), force_error["_errors"], np),
            "equal_or_lower_p99": bool(lerr["p99"] <= force_error["p99"]
                                       and lerr["p99_max"] <= force_error["p99_max"]),
            "stage_ms": {k[3:]: v for k, v in lacc.items()},
            "theta_ms_per_step": lacc["ms_theta"], "theta_share_of_step": lacc["ms_theta"] / lacc["ms_step"],
            "theta_ms_per_step_list": ltheta, "force_ms_per_step_list": lforce,
            "interactions_per_step": lerr["interactions"],
            "interaction_ratio_vs_plain": force_error["interactions"] / max(1.0, lerr["interactions"]),
            "theta_mean": float(th.mean()), "theta_p10": float(np.percentile(th, 10)),
            "theta_p90": float(np.percentile(th, 90)),
            "model": os.path.relpath(model_path, ROOT),
            "gint_per_s": lerr["interactions"] * (world if args.workload != "ensemble" else 1)
                          / (lms * 1e-3) / 1e9,
        }

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        os.environ.setdefault("OMP_NUM_THREADS", str(cores))
        sec, k, cpu_inter = cpu_step_time(arrs, counts, args)
        cpu = {"value": sec * 1e3, "unit": "ms/step", "cores": cores, "kind": "port",
               "sample": "%d full step(s) of the same %d-body %s workload after one warm-up step "
                         "(oracle/refbh.c, OpenMP force pass; tree stages serial%s)"
                         % (k, n, args.workload, "; one port instance per universe" if counts is not None else ""),
               "interactions_per_step": cpu_inter}

    # replicas (one independent universe per rank): time per universe-step of the job;
    # a sharded ensemble: the job's step takes the slowest rank's time
    replicas = args.workload != "ensemble"
    div = world if replicas else 1
    job_inter = interactions * world if replicas else reduce_sum(interactions, dist, dev)
    if force_error is not None:
        force_error.pop("_errors", None)
    if rank == 0:
        line = {
            "metric": METRIC, "value": ms / div, "unit": "ms/step", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
            "scaling": "weak" if replicas else "strong", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded %s, %d bodies %s" % (WORKLOADS[args.workload]["what"], n,
                                                            "per replica" if replicas else "on rank 0's shard"),
            "config": _config(args, n, counts),
            "gint_per_s": job_inter / (ms * 1e-3) / 1e9,
            "gint_per_s_force_only": inter_ts / (force_ms * 1e-3) / 1e9,
            "interactions_per_step": interactions,
            "max_depth": int(st["max_depth"]), "cells": cells,
            "build_contention": {"lock_waits": int(st["lock_waits"]), "cas_misses": int(st["cas_misses"])},
            "force_error": force_error,
            "stage_ms": {k[3:]: v for k, v in acc.items()},
            "stages": stages,
            "roofline": roofline,
            "autotune": None if tune is None else {k: tune[k] for k in (
                "force_threads", "stack_cap", "build_phases", "build_buckets", "top_phase", "vote_width", "max_depth",
                "ms_force",
                "ms_force_before",
                "ms_tree", "ms_tree_before")},
            "e2e": {"value": e2e_ms / div, "unit": "ms/step", "h2d_bytes_per_step": 36 * n,
                    "d2h_bytes_per_step": 36 * n, "wall_ms_per_step": wall_ms,
                    "path": "nbh_step_io: pinned host arrays in, one step, pinned host arrays out, one wait",
                    "three_calls": e2e_three},
            "gpu_launches": graph_launches(**({"build_phases": tune["build_phases"], "build_buckets": tune["build_buckets"]}
                                              if tune else {})) * args.steps,
            "clocks": clock_info,
            "cpu_baseline": cpu,
            "learned_theta": learned,
        }
        print(json.dumps(line))
    sim.close()
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
