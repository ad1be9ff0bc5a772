"""ctypes bindings of libnbh.so (include/nbh.h).

The library is built in-tree (gpu-nbody_gb300/nbh/libnbh.so) by nbh.build; importing
this module loads it and fails loudly if it is missing.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libnbh.so")

NBH_ABI_VERSION = 1
NBH_OK = 0
NBH_ERR_INVALID = -1
NBH_ERR_CUDA = -2
NBH_ERR_POOL = -3
NBH_ERR_DEPTH = -4
NBH_ERR_TIMEOUT = -5
NBH_ERR_STATE = -6
NBH_ERR_NOMEM = -7
NBH_ERR_NODEVICE = -8
NBH_ERR_MODEL = -9
NBH_MAXDEPTH = 64
NBH_ARITH_FMA = 0
NBH_ARITH_REFERENCE = 1
NBH_MLP_PARAMS = 5057
NBH_MLP_FEATURES = 12
NBH_DIRECT_STATIC_MAX = 65536

ERROR_NAMES = {
    NBH_OK: "NBH_OK", NBH_ERR_INVALID: "NBH_ERR_INVALID", NBH_ERR_CUDA: "NBH_ERR_CUDA",
    NBH_ERR_POOL: "NBH_ERR_POOL", NBH_ERR_DEPTH: "NBH_ERR_DEPTH", NBH_ERR_TIMEOUT: "NBH_ERR_TIMEOUT",
    NBH_ERR_STATE: "NBH_ERR_STATE", NBH_ERR_NOMEM: "NBH_ERR_NOMEM", NBH_ERR_NODEVICE: "NBH_ERR_NODEVICE",
    NBH_ERR_MODEL: "NBH_ERR_MODEL",
}


class NbhConfig(C.Structure):
    _fields_ = [
        ("abi_version", C.c_int32), ("device", C.c_int32),
        ("theta", C.c_float), ("eps", C.c_float), ("theta2", C.c_float), ("eps2", C.c_float),
        ("dt", C.c_float), ("G", C.c_float), ("pool_factor", C.c_float),
        ("vote_width", C.c_int32), ("arith", C.c_int32), ("precise", C.c_int32),
        ("stage_timing", C.c_int32), ("use_graph", C.c_int32), ("force_threads", C.c_int32),
        ("stack_cap", C.c_int32), ("build_phases", C.c_int32), ("build_buckets", C.c_int32),
        ("top_phase", C.c_int32), ("force_list", C.c_int32), ("reserved", C.c_int32 * 2),
    ]


class NbhStats(C.Structure):
    _fields_ = [
        ("steps", C.c_int64), ("interactions", C.c_int64),
        ("max_depth", C.c_int32), ("cells", C.c_int32), ("nuniverses", C.c_int32),
        ("nbodies", C.c_int32), ("pool_nodes", C.c_int32), ("status", C.c_int32),
        ("lock_waits", C.c_int32), ("cas_misses", C.c_int32),
        ("ms_bbox", C.c_float), ("ms_build", C.c_float), ("ms_summarize", C.c_float),
        ("ms_sort", C.c_float), ("ms_force", C.c_float), ("ms_integrate", C.c_float),
        ("ms_step", C.c_float), ("ms_theta", C.c_float), ("reserved", C.c_float * 7),
    ]


class NbhDiag(C.Structure):
    _fields_ = [
        ("mass", C.c_double), ("com", C.c_double * 3), ("momentum", C.c_double * 3),
        ("angular_momentum", C.c_double * 3), ("kinetic", C.c_double), ("potential", C.c_double),
        ("potential_unsoftened", C.c_double), ("max_depth", C.c_int32), ("has_potential", C.c_int32),
    ]


NBH_DIAG_POTENTIAL = 1
NBH_TUNE_VOTE = 1
NBH_TUNE_MAX_TRIALS = 64


class NbhTune(C.Structure):
    _fields_ = [
        ("force_threads", C.c_int32), ("stack_cap", C.c_int32), ("build_phases", C.c_int32),
        ("build_buckets", C.c_int32), ("vote_width", C.c_int32), ("max_depth", C.c_int32),
        ("ms_force", C.c_float), ("ms_force_before", C.c_float),
        ("ms_tree", C.c_float), ("ms_tree_before", C.c_float), ("trials", C.c_int32),
        ("trial_kind", C.c_int32 * NBH_TUNE_MAX_TRIALS), ("trial_a", C.c_int32 * NBH_TUNE_MAX_TRIALS),
        ("trial_b", C.c_int32 * NBH_TUNE_MAX_TRIALS), ("trial_vote", C.c_int32 * NBH_TUNE_MAX_TRIALS),
        ("trial_ms", C.c_float * NBH_TUNE_MAX_TRIALS), ("top_phase", C.c_int32),
    ]


class NbhHostState(C.Structure):
    _fields_ = [(k, C.c_void_p) for k in ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az")]


_P = C.c_void_p
_F = C.POINTER(C.c_float)
_I = C.POINTER(C.c_int32)
_D = C.POINTER(C.c_double)

# name: (restype, argtypes)
SIGNATURES = {
    "nbh_config_default": (None, [C.POINTER(NbhConfig)]),
    "nbh_create": (C.c_int, [C.POINTER(NbhConfig), C.POINTER(_P)]),
    "nbh_destroy": (C.c_int, [_P]),
    "nbh_load": (C.c_int, [_P, C.c_int32] + [_P] * 7),
    "nbh_load_batch": (C.c_int, [_P, C.c_int32, _P] + [_P] * 7),
    "nbh_step": (C.c_int, [_P, C.c_int32]),
    "nbh_step_async": (C.c_int, [_P, C.c_int32]),
    "nbh_synchronize": (C.c_int, [_P]),
    "nbh_read": (C.c_int, [_P] + [_P] * 9),
    "nbh_write": (C.c_int, [_P] + [_P] * 9),
    "nbh_step_io": (C.c_int, [_P, C.c_int32, C.POINTER(NbhHostState), C.POINTER(NbhHostState)]),
    "nbh_get_stats": (C.c_int, [_P, C.POINTER(NbhStats)]),
    "nbh_get_number_of_bodies": (C.c_int32, [_P]),
    "nbh_export_float4": (C.c_int, [_P, _P, _P]),
    "nbh_last_error_message": (C.c_char_p, [_P]),
    "nbh_get_stream": (C.c_void_p, [_P]),
    "nbh_selftest_wait": (C.c_int, [C.c_int32, C.c_int64, _I]),
    "nbh_measure_fp32_peak": (C.c_int, [C.c_int32, _D]),
    "nbh_last_error": (C.c_int, [_P]),
    "nbh_number_of_nodes": (C.c_int32, [C.c_int32, C.c_float]),
    "nbh_read_tree": (C.c_int, [_P] + [_P] * 8),
    "nbh_direct_f64": (C.c_int, [_P, C.c_int32, _P, _P, _P, _P]),
    "nbh_direct_f64_static": (C.c_int, [_P, C.c_int32, _P, _P, _P, _P]),
    "nbh_diagnostics": (C.c_int, [_P, C.c_int32, C.POINTER(NbhDiag), C.c_int32]),
    "nbh_autotune": (C.c_int, [_P, C.c_int32, C.POINTER(NbhTune)]),
    "nbh_generate_uniform_ball": (C.c_int, [C.c_uint64, C.c_int32, C.c_int32, C.c_float, C.c_float] + [_P] * 7),
    "nbh_generate_plummer": (C.c_int, [C.c_uint64, C.c_int32, C.c_int32, C.c_float, C.c_float] + [_P] * 7),
    "nbh_generate_disc": (C.c_int, [C.c_uint64, C.c_int32, C.c_int32, C.c_float, C.c_float, C.c_float,
                                    C.c_float] + [_P] * 7),
    "nbh_generate_random_cube": (C.c_int, [C.c_uint64, C.c_int32, C.c_int32, C.c_float] + [_P] * 4),
    "nbh_generate_sphere_surface": (C.c_int, [C.c_uint64, C.c_int32, C.c_int32] + [_P] * 4),
    "nbh_generate_fibonacci_sphere": (C.c_int, [C.c_uint64, C.c_int32, C.c_int32] + [_P] * 4),
    "nbh_generate_lonlat_sphere": (C.c_int, [C.c_uint64, C.c_int32, C.c_int32] + [_P] * 4),
    "nbh_generate_rotating_disk": (C.c_int, [C.c_uint64, C.c_int32, C.c_int32, C.c_float, C.c_float,
                                             C.c_float] + [_P] * 7),
    "nbh_set_theta_model": (C.c_int, [_P, _P, C.c_int32, _P, _P, C.c_float, C.c_float, C.c_int32]),
    "nbh_set_theta_interval": (C.c_int, [_P, C.c_int32]),
    "nbh_set_theta_grouping": (C.c_int, [_P, C.c_int32]),
    "nbh_read_theta": (C.c_int, [_P, _P]),
    "nbh_force_probe": (C.c_int, [_P, _P, _P, _P, _P, _P, C.POINTER(C.c_int64)]),
    "nbh_theta_features": (C.c_int, [_P, _P, C.c_int32]),
    "nbh_mlp_train": (C.c_int, [C.c_int32, _P, _P, _P, C.c_int32, C.c_float, C.c_int32, C.c_float, _F]),
    "nbh_mlp_grad": (C.c_int, [C.c_int32, _P, _P, _P, C.c_int32, C.c_float, _P, _F]),
    "nbh_mlp_forward": (C.c_int, [C.c_int32, _P, _P, C.c_int32, _P]),
    "nbh_universe_read": (C.c_int, [C.c_char_p, _I] + [_P] * 7),
    "nbh_universe_write": (C.c_int, [C.c_char_p, C.c_int32] + [_P] * 7),
}

_lib = None


def load(path: str | None = None):
    """Load libnbh.so (building it first if the sources are newer).  Raises if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        try:
            from . import build as _build
            _build.build()
        except Exception as e:  # noqa: BLE001
            raise ImportError("libnbh.so is not built and building it failed: %s" % e) from e
    if not os.path.exists(p):
        raise ImportError("libnbh.so not found at %s (run nbh.build.build())" % p)
    L = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = L
    return L


class NbhError(RuntimeError):
    def __init__(self, code: int, message: str):
        self.code = code
        super().__init__("%s (%d): %s" % (ERROR_NAMES.get(code, "NBH_ERR"), code, message))


def check(code: int, sim_handle=None) -> int:
    if code != NBH_OK:
        msg = load().nbh_last_error_message(sim_handle)
        raise NbhError(code, msg.decode() if msg else "")
    return code
