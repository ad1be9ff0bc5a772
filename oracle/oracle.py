"""ctypes front end of the oracle (test infrastructure only).

``Oracle`` wraps oracle/refbh.c (the CPU restatement of the reference step);
``run_reference`` runs the reference project's own kernels compiled as C++ (only where
the reference sources are mounted, see oracle/build.py).  Only tests/,
__graft_entry__.smoke and bench.py's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import build as _build  # noqa: E402

_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")

RB_MAXDEPTH = 64


class _RbSim(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("nn", C.c_int),
        ("theta2", C.c_float), ("eps2", C.c_float), ("dt", C.c_float), ("G", C.c_float),
        ("vote", C.c_int), ("fma", C.c_int), ("precise", C.c_int),
        ("x", C.POINTER(C.c_float)), ("y", C.POINTER(C.c_float)),
        ("z", C.POINTER(C.c_float)), ("m", C.POINTER(C.c_float)),
        ("vx", C.POINTER(C.c_float)), ("vy", C.POINTER(C.c_float)), ("vz", C.POINTER(C.c_float)),
        ("ax", C.POINTER(C.c_float)), ("ay", C.POINTER(C.c_float)), ("az", C.POINTER(C.c_float)),
        ("kx", C.POINTER(C.c_float)), ("ky", C.POINTER(C.c_float)), ("kz", C.POINTER(C.c_float)),
        ("kvx", C.POINTER(C.c_float)), ("kvy", C.POINTER(C.c_float)), ("kvz", C.POINTER(C.c_float)),
        ("theta_body", C.POINTER(C.c_float)), ("ebound", C.POINTER(C.c_float)),
        ("child", C.POINTER(C.c_int)), ("count", C.POINTER(C.c_int)),
        ("start", C.POINTER(C.c_int)), ("sorted", C.POINTER(C.c_int)),
        ("radius", C.c_float),
        ("bottom", C.c_int), ("maxdepth", C.c_int), ("step", C.c_int), ("error", C.c_int),
        ("interactions", C.c_longlong),
        ("theta_group", C.c_int),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(path)
        P = C.POINTER(_RbSim)
        L.rb_number_of_nodes.argtypes = [C.c_int, C.c_float]
        L.rb_number_of_nodes.restype = C.c_int
        L.rb_create.argtypes = [C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float,
                                C.c_int, C.c_int, C.c_int]
        L.rb_create.restype = P
        L.rb_destroy.argtypes = [P]
        L.rb_load.argtypes = [P] + [C.c_void_p] * 7
        L.rb_set_theta_body.argtypes = [P, C.c_void_p]
        L.rb_enable_ebound.argtypes = [P, C.c_int]
        L.rb_set_theta_group.argtypes = [P, C.c_int]
        for fn in ("rb_bbox", "rb_build", "rb_summarize", "rb_sort", "rb_force",
                   "rb_integrate", "rb_step", "rb_tree"):
            getattr(L, fn).argtypes = [P]
            getattr(L, fn).restype = C.c_int
        L.rb_direct_f64.argtypes = [C.c_int, _f32p, _f32p, _f32p, _f32p, C.c_double, C.c_double,
                                    C.c_int, _i32p, _f64p, _f64p, _f64p]
        _lib = L
    return _lib


def number_of_nodes(n: int, pool_factor: float = 2.0) -> int:
    return lib().rb_number_of_nodes(int(n), float(pool_factor))


def _arr(ptr, count, dtype):
    return np.ctypeslib.as_array(ptr, shape=(count,)).astype(dtype, copy=True)


class Oracle:
    """One universe stepped by the CPU restatement.

    theta/eps are the opening angle and softening length; their float32 squares are
    used unless theta2/eps2 give the squares verbatim (the reference's THETA and EPSILON
    macros, e.g. 1.5 and 0.0025).  vote = bodies voting together (16: reference
    work-group, 32: one CUDA warp); fma = 1 fuses a*b+c, 0 rounds the product first.
    """

    def __init__(self, n, theta=0.5, eps=0.05, dt=0.025, G=1.0, vote=32, fma=True,
                 precise=False, pool_factor=2.0, nn=None, theta2=None, eps2=None):
        self.n = int(n)
        self.nn = int(nn) if nn is not None else number_of_nodes(self.n, pool_factor)
        t2 = np.float32(theta2) if theta2 else np.float32(theta) * np.float32(theta)
        e2 = np.float32(eps2) if eps2 else np.float32(eps) * np.float32(eps)
        self.eps2 = float(e2)
        self._p = lib().rb_create(self.n, self.nn, float(t2), float(e2), dt, G, int(vote),
                                  int(bool(fma)), int(bool(precise)))
        if not self._p:
            raise ValueError("rb_create failed")

    def __del__(self):
        p = getattr(self, "_p", None)
        if p:
            lib().rb_destroy(p)
            self._p = None

    @property
    def s(self):
        return self._p.contents

    def load(self, x, y, z, vx, vy, vz, m):
        arrs = [np.ascontiguousarray(a, dtype=np.float32) if a is not None else None
                for a in (x, y, z, vx, vy, vz, m)]
        self._keep = arrs
        ptrs = [a.ctypes.data if a is not None else None for a in arrs]
        lib().rb_load(self._p, *ptrs)

    def set_theta_body(self, theta):
        if theta is None:
            lib().rb_set_theta_body(self._p, None)
        else:
            t = np.ascontiguousarray(theta, dtype=np.float32)
            assert t.shape == (self.n,)
            lib().rb_set_theta_body(self._p, t.ctypes.data)

    def set_theta_group(self, on=True):
        lib().rb_set_theta_group(self._p, int(bool(on)))

    def enable_ebound(self, on=True):
        lib().rb_enable_ebound(self._p, int(bool(on)))

    def ebound(self):
        return _arr(self.s.ebound, self.n, np.float32)

    def _call(self, fn):
        return getattr(lib(), fn)(self._p)

    def bbox(self): return self._call("rb_bbox")
    def build(self): return self._call("rb_build")
    def summarize(self): return self._call("rb_summarize")
    def sort(self): return self._call("rb_sort")
    def force(self): return self._call("rb_force")
    def integrate(self): return self._call("rb_integrate")
    def tree(self): return self._call("rb_tree")

    def step(self, nsteps=1):
        for _ in range(nsteps):
            e = self._call("rb_step")
            if e:
                return e
        return 0

    def state(self):
        s, n = self.s, self.n
        return {k: _arr(getattr(s, k), n, np.float32)
                for k in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az")} | {
            "m": _arr(s.m, n, np.float32)}

    def tree_arrays(self):
        s, nn = self.s, self.nn
        return {
            "child": _arr(s.child, 8 * (nn + 1), np.int32).reshape(nn + 1, 8),
            "count": _arr(s.count, nn + 1, np.int32),
            "start": _arr(s.start, nn + 1, np.int32),
            "sorted": _arr(s.sorted, self.n, np.int32),
            "x": _arr(s.x, nn + 1, np.float32), "y": _arr(s.y, nn + 1, np.float32),
            "z": _arr(s.z, nn + 1, np.float32), "m": _arr(s.m, nn + 1, np.float32),
            "bottom": s.bottom, "radius": s.radius, "maxdepth": s.maxdepth,
        }

    @property
    def interactions(self):
        return self.s.interactions

    @property
    def maxdepth(self):
        return self.s.maxdepth

    @property
    def error(self):
        return self.s.error


def direct_f64(x, y, z, m, eps, idx, G=1.0, eps2=None):
    """FP64 direct-sum accelerations of bodies idx.  The softening is eps2 if given, else
    the float32 square of eps (the value the GPU step uses)."""
    f = [np.ascontiguousarray(a, dtype=np.float32) for a in (x, y, z, m)]
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    k = idx.size
    ax, ay, az = (np.zeros(k, np.float64) for _ in range(3))
    e2 = float(eps2) if eps2 is not None else float(np.float32(eps) * np.float32(eps))
    lib().rb_direct_f64(f[0].size, f[0], f[1], f[2], f[3], e2, float(G), k, idx, ax, ay, az)
    return ax, ay, az


def diagnostics_f64(x, y, z, vx, vy, vz, m, eps, G=1.0, potential=True, block=2048):
    """FP64 restatement of nbh_diagnostics for one universe: mass, centre of mass, momentum
    (printImpulse, GPUBarnesHutNBodySimulation.java:347-365), angular momentum, kinetic energy
    (:318-324) and the pair potentials -G sum_{i<j} m_i m_j / sqrt(r^2 + eps^2) and
    -G sum_{i<j} m_i m_j / r (each pair once; see reference_energy for :326-335)."""
    x, y, z, vx, vy, vz, m = (np.asarray(a, dtype=np.float64) for a in (x, y, z, vx, vy, vz, m))
    M = m.sum()
    out = {"mass": M, "com": [float((m * x).sum() / M), float((m * y).sum() / M), float((m * z).sum() / M)],
           "momentum": [float((m * vx).sum()), float((m * vy).sum()), float((m * vz).sum())],
           "angular_momentum": [float((m * (y * vz - z * vy)).sum()), float((m * (z * vx - x * vz)).sum()),
                                float((m * (x * vy - y * vx)).sum())],
           "kinetic": float((0.5 * m * (vx * vx + vy * vy + vz * vz)).sum())}
    if potential:
        n = x.size
        ps = pu = 0.0
        e2 = float(np.float32(eps) * np.float32(eps))
        for a in range(0, n, block):
            b = min(n, a + block)
            dx = x[a:b, None] - x[None, :]
            dy = y[a:b, None] - y[None, :]
            dz = z[a:b, None] - z[None, :]
            r2 = dx * dx + dy * dy + dz * dz
            mm = m[a:b, None] * m[None, :]
            self_ = np.arange(a, b)[:, None] == np.arange(n)[None, :]
            with np.errstate(divide="ignore"):
                ps += np.where(self_, 0.0, mm / np.sqrt(r2 + e2)).sum()
                pu += np.where(self_, 0.0, mm / np.sqrt(r2)).sum()
        out["potential"] = -0.5 * G * ps
        out["potential_unsoftened"] = -0.5 * G * pu
    return out


def reference_energy(x, y, z, vx, vy, vz, m):
    """printEnergy (GPUBarnesHutNBodySimulation.java:305-339) as the reference computes it:
    ekin = sum m v^2 / 2 with v = |v| (:318-324); epot = sum_{i<j} 2 m_i m_j / r, each pair
    added twice (:326-335); etot = ekin - epot (:338).  Small N only (pairwise loop)."""
    x, y, z, vx, vy, vz, m = (np.asarray(a, dtype=np.float64) for a in (x, y, z, vx, vy, vz, m))
    ekin = epot = 0.0
    n = x.size
    for i in range(n):
        v = np.sqrt(vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i])
        ekin += m[i] * v * v / 2
        for j in range(i + 1, n):
            r = np.sqrt((x[i] - x[j]) ** 2 + (y[i] - y[j]) ** 2 + (z[i] - z[j]) ** 2)
            epot += 2 * (m[i] * m[j]) / r
    return {"ekin": ekin, "epot": epot, "etot": ekin - epot}


def rel_force_error(ax, ay, az, rx, ry, rz):
    """|a - a_ref| / |a_ref| per body."""
    num = np.sqrt((ax - rx) ** 2 + (ay - ry) ** 2 + (az - rz) ** 2)
    den = np.sqrt(rx ** 2 + ry ** 2 + rz ** 2)
    return num / np.maximum(den, 1e-300)


# ---------------------------------------------------------------------------------------
# The reference's own kernels (compiled as C++; available only where the sources are).

def reference_available() -> bool:
    return _build.reference_available()


def run_reference(x, y, z, vx, vy, vz, m, nsteps):
    """Run the reference kernels for nsteps from the given state.

    The reference fixes THETA = 1.5 (theta^2), EPSILON = 0.0025 (eps^2) and
    TIMESTEP = 0.025 at compile time (calculateforce.cl:13-18, integrate.cl:12).
    Returns per-step arrays [nsteps, n] and the final sorted order / info."""
    n = int(np.asarray(x).size)
    path = _build.build_reference(n)
    L = C.CDLL(path)
    L.ref_run.argtypes = [C.c_void_p] * 7 + [C.c_int] + [C.c_void_p] * 12
    L.ref_run.restype = C.c_int
    ins = [np.ascontiguousarray(a, dtype=np.float32) for a in (x, y, z, vx, vy, vz, m)]
    outs = {k: np.zeros((nsteps, n), np.float32)
            for k in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az")}
    sorted_ = np.zeros(n, np.int32)
    info = np.zeros(5, np.int32)
    root = np.zeros(5, np.float32)
    err = L.ref_run(*[a.ctypes.data for a in ins], int(nsteps),
                    *[outs[k].ctypes.data for k in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az")],
                    sorted_.ctypes.data, info.ctypes.data, root.ctypes.data)
    return {"error": err, "sorted": sorted_, "maxdepth": int(info[0]), "bottom": int(info[1]),
            "step": int(info[3]), "root_count": int(info[4]), "root": root, **outs}


# Compile-time constants of the reference kernels (calculateforce.cl:14-18, integrate.cl:12).
REFERENCE_THETA2 = 1.5      # THETA is theta^2
REFERENCE_EPS2 = 0.0025     # EPSILON is eps^2
REFERENCE_DT = 0.025
