"""nbh — GB300-native Barnes-Hut step engine (host side over libnbh.so's C ABI).

The hot path (bounding box, octree build, summarize, sort, force, integrate) runs as
hand-written sm_103a CUDA kernels in libnbh.so; this package only marshals arrays.
Importing it loads libnbh.so and raises ImportError if the library is missing.
"""
from . import _lib
from ._lib import NbhError, NBH_ARITH_FMA, NBH_ARITH_REFERENCE  # noqa: F401
from .simulation import GPUBarnesHutNBodySimulation, Mode, Simulation, make_config  # noqa: F401
from . import universe  # noqa: F401

_lib.load()
