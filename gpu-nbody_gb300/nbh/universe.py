"""Universe generators with the reference's interface (universe/UniverseGenerator.java:22):
``generate(offset, nbodies, x, y, z, vx, vy, vz, m)`` fills caller-owned float32 arrays.

Each class maps to one reference generator; all are seeded (the reference uses
Math.random()) and run in libnbh's host code.  ``SerializedUniverseGenerator`` and
``write_universe`` read and write the reference's .universe files.
"""
from __future__ import annotations

import numpy as np

from . import _lib as L


def _p(a):
    if a is None:
        return None
    if a.dtype != np.float32 or not a.flags.c_contiguous:
        raise TypeError("generator outputs must be contiguous float32 arrays")
    return a.ctypes.data


class UniverseGenerator:
    def generate(self, offset, nbodies, x, y, z, vx, vy, vz, m):  # pragma: no cover - interface
        raise NotImplementedError

    def arrays(self, nbodies):
        """Convenience: allocate and fill (x, y, z, vx, vy, vz, m)."""
        out = [np.zeros(nbodies, np.float32) for _ in range(7)]
        self.generate(0, nbodies, *out)
        return out


class UniformBallUniverseGenerator(UniverseGenerator):
    """Uniform in a ball, Gaussian velocities, masses 1/n (the 16,384-body workload)."""

    def __init__(self, seed=1, radius=1.0, vsigma=0.05):
        self.seed, self.radius, self.vsigma = seed, radius, vsigma

    def generate(self, offset, nbodies, x, y, z, vx, vy, vz, m):
        L.check(L.load().nbh_generate_uniform_ball(self.seed, offset, nbodies, self.radius, self.vsigma,
                                                   _p(x), _p(y), _p(z), _p(vx), _p(vy), _p(vz), _p(m)))


class PlummerUniverseGenerator(UniverseGenerator):
    """PlummerUniverseGenerator.java:6-43, scale radius a and mass M (no 3*pi/16 rescale)."""

    def __init__(self, seed=1, a=1.0, M=1.0):
        self.seed, self.a, self.M = seed, a, M

    def generate(self, offset, nbodies, x, y, z, vx, vy, vz, m):
        L.check(L.load().nbh_generate_plummer(self.seed, offset, nbodies, self.a, self.M,
                                              _p(x), _p(y), _p(z), _p(vx), _p(vy), _p(vz), _p(m)))


class DiscGalaxyGenerator(UniverseGenerator):
    """Exponential disc + central point mass + Plummer halo (the 4M-body precision case)."""

    def __init__(self, seed=1, rd=1.0, zd=0.1, center_mass=0.1, halo_frac=0.1):
        self.seed, self.rd, self.zd, self.mc, self.hf = seed, rd, zd, center_mass, halo_frac

    def generate(self, offset, nbodies, x, y, z, vx, vy, vz, m):
        L.check(L.load().nbh_generate_disc(self.seed, offset, nbodies, self.rd, self.zd, self.mc, self.hf,
                                           _p(x), _p(y), _p(z), _p(vx), _p(vy), _p(vz), _p(m)))


class RandomCubicUniverseGenerator(UniverseGenerator):
    """RandomCubicUniverseGenerator.java:5-18."""

    def __init__(self, range_, seed=1):
        self.range, self.seed = range_, seed

    def generate(self, offset, nbodies, x, y, z, vx, vy, vz, m):
        L.check(L.load().nbh_generate_random_cube(self.seed, offset, nbodies, self.range,
                                                  _p(x), _p(y), _p(z), _p(m)))


class SphericalUniverseGenerator(UniverseGenerator):
    """SphericalUniverseGenerator.java:6-20."""

    def __init__(self, seed=1):
        self.seed = seed

    def generate(self, offset, nbodies, x, y, z, vx, vy, vz, m):
        L.check(L.load().nbh_generate_sphere_surface(self.seed, offset, nbodies, _p(x), _p(y), _p(z), _p(m)))


class MonteCarloSphericalUniverseGenerator(UniverseGenerator):
    """MonteCarloSphericalUniverseGenerator.java:6-27 (Fibonacci sphere)."""

    def __init__(self, seed=1):
        self.seed = seed

    def generate(self, offset, nbodies, x, y, z, vx, vy, vz, m):
        L.check(L.load().nbh_generate_fibonacci_sphere(self.seed, offset, nbodies, _p(x), _p(y), _p(z), _p(m)))


class LonLatSphericalUniverseGenerator(UniverseGenerator):
    """LonLatSphericalUniverseGenerator.java:9-29."""

    def __init__(self, seed=1):
        self.seed = seed

    def generate(self, offset, nbodies, x, y, z, vx, vy, vz, m):
        L.check(L.load().nbh_generate_lonlat_sphere(self.seed, offset, nbodies, _p(x), _p(y), _p(z), _p(m)))


class RotatingDiskGalaxyGenerator(UniverseGenerator):
    """RotatingDiskGalaxyGenerator.java:5-43."""

    def __init__(self, r, velocity_multiplier, center_mass, seed=1):
        self.r, self.vmul, self.mc, self.seed = r, velocity_multiplier, center_mass, seed

    def generate(self, offset, nbodies, x, y, z, vx, vy, vz, m):
        L.check(L.load().nbh_generate_rotating_disk(self.seed, offset, nbodies, self.r, self.vmul, self.mc,
                                                    _p(x), _p(y), _p(z), _p(vx), _p(vy), _p(vz), _p(m)))


class SerializedUniverseGenerator(UniverseGenerator):
    """SerializedUniverseGenerator.java:13-56: reads a .universe file; generate() requires
    the same body count (:41-42)."""

    def __init__(self, path):
        import ctypes as C
        self.path = str(path)
        n = C.c_int32()
        lib = L.load()
        L.check(lib.nbh_universe_read(self.path.encode(), C.byref(n), None, None, None, None, None, None, None))
        self.nbodies = n.value
        self.data = [np.empty(self.nbodies, np.float32) for _ in range(7)]
        L.check(lib.nbh_universe_read(self.path.encode(), C.byref(n), *[a.ctypes.data for a in self.data]))

    def generate(self, offset, nbodies, x, y, z, vx, vy, vz, m):
        if nbodies != self.nbodies:
            raise ValueError("invalid amount of bodies for serialized universe")
        for dst, src in zip((x, y, z, vx, vy, vz, m), self.data):
            if dst is not None:
                dst[offset:offset + nbodies] = src


def write_universe(path, x, y, z, vx, vy, vz, m):
    """UniverseSerializer.java:25-34 (writeInt(n) then seven float[] objects)."""
    arr = [np.ascontiguousarray(a, dtype=np.float32) for a in (x, y, z, vx, vy, vz, m)]
    L.check(L.load().nbh_universe_write(str(path).encode(), arr[0].size, *[a.ctypes.data for a in arr]))
