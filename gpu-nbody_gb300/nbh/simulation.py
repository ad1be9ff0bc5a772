"""Host-side mirror of the reference's simulation API.

``GPUBarnesHutNBodySimulation`` keeps the names, argument meaning and call order of the
reference's AbstractNBodySimulation / GPUBarnesHutNBodySimulation
(src/ch/fhnw/woipv/nbody/simulation/AbstractNBodySimulation.java:5-44,
gpu/GPUBarnesHutNBodySimulation.java:104-151,229-271,376-379): construct with a mode, a
body count and a UniverseGenerator, ``init()``, ``initGLBuffers()``, then ``step()`` per
frame.  Every call goes through the C ABI of libnbh.so; the GL interop mode writes the
float4 vertex buffers into headless device buffers instead of GL VBOs.
"""
from __future__ import annotations

import ctypes as C
import enum

import numpy as np

from . import _lib as L


class Mode(enum.Enum):
    """AbstractNBodySimulation.Mode (:41-43)."""
    GL_INTEROP = 0
    DEFAULT = 1


def _ptr(a):
    return None if a is None else a.ctypes.data


def _f32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float32)


def make_config(theta=0.5, eps=0.05, dt=0.025, G=1.0, pool_factor=2.0, vote_width=None,
                arith=L.NBH_ARITH_FMA, precise=False, stage_timing=False, use_graph=True,
                device=0, theta2=0.0, eps2=0.0, force_threads=0, stack_cap=0, build_phases=0,
                build_buckets=0, top_phase=0, force_list=0) -> L.NbhConfig:
    cfg = L.NbhConfig()
    L.load().nbh_config_default(C.byref(cfg))
    cfg.device = device
    cfg.theta, cfg.eps, cfg.dt, cfg.G = theta, eps, dt, G
    cfg.theta2, cfg.eps2 = theta2, eps2
    cfg.pool_factor = pool_factor
    if vote_width is not None:          # None: the library default (64)
        cfg.vote_width = vote_width
    cfg.arith = arith
    cfg.precise = int(bool(precise))
    cfg.stage_timing = int(bool(stage_timing))
    cfg.use_graph = int(bool(use_graph))
    cfg.force_threads, cfg.stack_cap, cfg.build_phases = force_threads, stack_cap, build_phases
    cfg.build_buckets = build_buckets
    cfg.top_phase = top_phase
    cfg.force_list = force_list
    return cfg


class Simulation:
    """Thin owner of one nbh_sim handle (any number of universes)."""

    def __init__(self, config: L.NbhConfig | None = None, **kw):
        self._L = L.load()
        self.config = config if config is not None else make_config(**kw)
        h = C.c_void_p()
        code = self._L.nbh_create(C.byref(self.config), C.byref(h))
        if code != L.NBH_OK:
            raise L.NbhError(code, (self._L.nbh_last_error_message(None) or b"").decode())
        self._h = h
        self.n = 0
        self.counts = None

    # -- lifetime ----------------------------------------------------------------------
    def close(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.nbh_destroy(h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, code):
        return L.check(code, self._h)

    # -- data --------------------------------------------------------------------------
    def load(self, x, y, z, vx=None, vy=None, vz=None, m=None):
        arr = [_f32(a) for a in (x, y, z, vx, vy, vz, m)]
        n = arr[0].size
        self._check(self._L.nbh_load(self._h, n, *[_ptr(a) for a in arr]))
        self.n = n
        self.counts = np.array([n], np.int32)

    def load_batch(self, counts, x, y, z, vx=None, vy=None, vz=None, m=None):
        counts = np.ascontiguousarray(counts, dtype=np.int32)
        arr = [_f32(a) for a in (x, y, z, vx, vy, vz, m)]
        self._check(self._L.nbh_load_batch(self._h, counts.size, counts.ctypes.data,
                                           *[_ptr(a) for a in arr]))
        self.n = int(counts.sum())
        self.counts = counts

    def step(self, nsteps: int = 1):
        self._check(self._L.nbh_step(self._h, int(nsteps)))

    def step_async(self, nsteps: int = 1):
        self._check(self._L.nbh_step_async(self._h, int(nsteps)))

    def synchronize(self):
        self._check(self._L.nbh_synchronize(self._h))

    def read(self):
        out = {k: np.empty(self.n, np.float32) for k in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az")}
        self._check(self._L.nbh_read(self._h, *[out[k].ctypes.data for k in
                                                ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az")]))
        return out

    def read_into(self, x=None, y=None, z=None, vx=None, vy=None, vz=None, ax=None, ay=None, az=None):
        self._check(self._L.nbh_read(self._h, *[_ptr(a) for a in (x, y, z, vx, vy, vz, ax, ay, az)]))

    def write(self, x=None, y=None, z=None, vx=None, vy=None, vz=None, ax=None, ay=None, az=None):
        arr = [_f32(a) for a in (x, y, z, vx, vy, vz, ax, ay, az)]
        self._check(self._L.nbh_write(self._h, *[_ptr(a) for a in arr]))

    def step_io(self, nsteps=1, write=None, read=None):
        """nbh_step_io: `write` (dict of host arrays by component name, written before the
        steps) and `read` (dict of float32 arrays filled after them), one wait in all."""
        def state(d, conv):
            if d is None:
                return None, None
            arrs = {k: conv(v) for k, v in d.items()}
            bad = set(arrs) - {k for k, _ in L.NbhHostState._fields_}
            if bad:
                raise ValueError("unknown components %s" % sorted(bad))
            return L.NbhHostState(**{k: _ptr(a) for k, a in arrs.items()}), arrs

        def in_array(a):
            a = _f32(a)
            if a.size != self.n:
                raise ValueError("write arrays must have n elements")
            return a

        def out_array(a):
            if a.dtype != np.float32 or not a.flags.c_contiguous or a.size != self.n:
                raise ValueError("read arrays must be contiguous float32 of n elements")
            return a
        sin, keep_in = state(write, in_array)
        sout, keep_out = state(read, out_array)
        self._check(self._L.nbh_step_io(self._h, int(nsteps), C.byref(sin) if sin else None,
                                        C.byref(sout) if sout else None))
        del keep_in, keep_out

    def stats(self) -> dict:
        s = L.NbhStats()
        self._check(self._L.nbh_get_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in L.NbhStats._fields_ if k != "reserved"}

    def tree(self) -> dict:
        st = self.stats()
        nn, n = st["pool_nodes"], self.n
        nc = nn + 1 - n
        child = np.empty(8 * nc, np.int32)
        node4 = np.empty(4 * (nn + 1), np.float32)
        count = np.empty(nc, np.int32)
        start = np.empty(nc, np.int32)
        sorted_ = np.empty(n, np.int32)
        nu = len(self.counts)
        roots = np.empty(nu, np.int32)
        radius = np.empty(nu, np.float32)
        bottom = C.c_int32()
        self._check(self._L.nbh_read_tree(self._h, child.ctypes.data, node4.ctypes.data, count.ctypes.data,
                                          start.ctypes.data, sorted_.ctypes.data, roots.ctypes.data,
                                          radius.ctypes.data, C.addressof(bottom)))
        return {"child": child.reshape(nc, 8), "node4": node4.reshape(nn + 1, 4), "count": count,
                "start": start, "sorted": sorted_, "roots": roots, "radius": radius,
                "bottom": bottom.value, "nnodes": nn, "nbody": n}

    def direct_f64(self, idx):
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        out = [np.empty(idx.size, np.float64) for _ in range(3)]
        self._check(self._L.nbh_direct_f64(self._h, idx.size, idx.ctypes.data, *[o.ctypes.data for o in out]))
        return out

    def diagnostics(self, potential: bool = False) -> list:
        """Per-universe mass, centre of mass, momentum, angular momentum, kinetic and (with
        potential=True, O(N^2)) potential energy, reduced on the GPU in FP64 (nbh_diagnostics)."""
        nu = 1 if self.counts is None else len(self.counts)
        arr = (L.NbhDiag * nu)()
        got = self._L.nbh_diagnostics(self._h, L.NBH_DIAG_POTENTIAL if potential else 0, arr, nu)
        if got < 0:
            self._check(got)
        out = []
        for d in arr[:got]:
            r = {"mass": d.mass, "com": list(d.com), "momentum": list(d.momentum),
                 "angular_momentum": list(d.angular_momentum), "kinetic": d.kinetic, "max_depth": d.max_depth}
            if d.has_potential:
                r.update({"potential": d.potential, "potential_unsoftened": d.potential_unsoftened,
                          "total": d.kinetic + d.potential})
            out.append(r)
        return out

    def autotune(self, vote: bool = False) -> dict:
        """Pick the force launch geometry and the build's insertion phases by timing them on
        the loaded universes (nbh_autotune); later steps use the choice.  vote=True also
        times vote widths 32 and 64 (changes the interaction set)."""
        t = L.NbhTune()
        self._check(self._L.nbh_autotune(self._h, L.NBH_TUNE_VOTE if vote else 0, C.byref(t)))
        trials = [{"kind": ("force", "tree")[t.trial_kind[k]], "a": t.trial_a[k], "b": t.trial_b[k],
                   "vote": t.trial_vote[k], "ms": t.trial_ms[k]} for k in range(t.trials)]
        return {"force_threads": t.force_threads, "stack_cap": t.stack_cap, "build_phases": t.build_phases,
                "build_buckets": t.build_buckets, "top_phase": t.top_phase, "vote_width": t.vote_width,
                "max_depth": t.max_depth, "ms_force": t.ms_force, "ms_force_before": t.ms_force_before,
                "ms_tree": t.ms_tree, "ms_tree_before": t.ms_tree_before, "trials": trials}

    def export_float4(self, dev_pos4: int | None, dev_vel4: int | None):
        self._check(self._L.nbh_export_float4(self._h, dev_pos4, dev_vel4))

    @property
    def stream(self) -> int:
        """cudaStream_t of this sim as an integer (torch.cuda.ExternalStream accepts it)."""
        return int(self._L.nbh_get_stream(self._h) or 0)

    @property
    def number_of_bodies(self) -> int:
        return int(self._L.nbh_get_number_of_bodies(self._h))


class GPUBarnesHutNBodySimulation:
    """Drop-in for the reference's GPUBarnesHutNBodySimulation (same life cycle)."""

    def __init__(self, mode: Mode, nbodies: int, generator, config: L.NbhConfig | None = None, **kw):
        self.mode = mode
        self.nbodies = int(nbodies)
        self.universe_generator = generator
        self._config = config
        self._kw = kw
        self.sim = None
        self._pos4 = None
        self._vel4 = None

    def init(self, gl=None):
        """Create the device state and load the generated universe (:110-151)."""
        n = self.nbodies
        arrays = [np.zeros(n, np.float32) for _ in range(7)]
        self.universe_generator.generate(0, n, *arrays)
        self.sim = Simulation(self._config, **self._kw)
        self.sim.load(*arrays)

    def initGLBuffers(self, gl=None, positionVBO: int = -1, velocityVBO: int = -1):  # noqa: N802
        """Headless vertex buffers (:229-246): two device float4[N] buffers that step()
        fills in GL_INTEROP mode, like copyVertices (copyvertices.cl:14-17)."""
        import torch  # device memory plumbing only
        self._pos4 = torch.empty((self.nbodies, 4), dtype=torch.float32, device="cuda")
        self._vel4 = torch.empty((self.nbodies, 4), dtype=torch.float32, device="cuda")

    @property
    def position_buffer(self):
        return self._pos4

    @property
    def velocity_buffer(self):
        return self._vel4

    def step(self):
        """One step (:248-271); in GL_INTEROP mode also refresh the vertex buffers."""
        self.sim.step(1)
        if self.mode == Mode.GL_INTEROP and self._pos4 is not None:
            self.sim.export_float4(self._pos4.data_ptr(), self._vel4.data_ptr())

    def getNumberOfBodies(self) -> int:  # noqa: N802
        return self.nbodies

    def close(self):
        if self.sim is not None:
            self.sim.close()
            self.sim = None
