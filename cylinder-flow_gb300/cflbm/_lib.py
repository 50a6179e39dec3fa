"""ctypes binding of include/cflbm.h (the solver's C ABI).

Loads the in-tree ``libcflbm.so``.  There is no fallback: if the library is
missing or fails to load, importing this module raises, so a GPU run can never
silently route around the CUDA kernels.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libcflbm.so")

D2Q9, D3Q27 = 9, 27
STORE_FP64, STORE_FP32, STORE_FP16DEV = 0, 1, 2
COMPUTE_FP64, COMPUTE_FP32, COMPUTE_DF64 = 0, 1, 2
PROFILE_CHANNEL, PROFILE_REF2D, PROFILE_REF3D, PROFILE_REF2DS = 0, 1, 2, 3
WALL_FREESLIP, WALL_NOSLIP, WALL_PERIODIC = 0, 1, 2
GEOM_NONE, GEOM_CYLINDER, GEOM_SPHERE = 0, 1, 2
LAYOUT_SOA, LAYOUT_ROWS = 0, 1
ROUND_NEAREST, ROUND_STOCHASTIC = 0, 1

ERRORS = {1: "invalid argument", 2: "CUDA error", 3: "out of memory", 4: "numeric error",
          5: "I/O error", 6: "unsupported"}

_dp = ctypes.POINTER(ctypes.c_double)


class Config(ctypes.Structure):
    _fields_ = [
        ("lattice", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int),
        ("nz", ctypes.c_int), ("storage", ctypes.c_int), ("compute", ctypes.c_int),
        ("profile", ctypes.c_int), ("wall_y", ctypes.c_int), ("wall_z", ctypes.c_int),
        ("tau0", ctypes.c_double), ("u0", ctypes.c_double), ("geom", ctypes.c_int),
        ("cx", ctypes.c_double), ("cy", ctypes.c_double), ("cz", ctypes.c_double),
        ("diam", ctypes.c_double), ("perturb_amp", ctypes.c_double),
        ("seed", ctypes.c_uint64), ("solid", ctypes.POINTER(ctypes.c_uint8)),
        ("alpha", _dp), ("ref_ran", ctypes.POINTER(ctypes.c_int32)),
        ("force_history", ctypes.c_int), ("device", ctypes.c_int), ("layout", ctypes.c_int),
        ("rounding", ctypes.c_int),
    ]


class Info(ctypes.Structure):
    _fields_ = [
        ("lattice", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int),
        ("nz", ctypes.c_int), ("storage", ctypes.c_int), ("compute", ctypes.c_int),
        ("profile", ctypes.c_int), ("ghost", ctypes.c_int), ("pitch_x", ctypes.c_int),
        ("pop_stride", ctypes.c_int64), ("steps_done", ctypes.c_int64),
        ("n_links", ctypes.c_int64), ("n_solid", ctypes.c_int64), ("omega", ctypes.c_double),
        ("bytes_per_cell_step", ctypes.c_double), ("device_bytes", ctypes.c_size_t),
        ("layout", ctypes.c_int),
    ]


class BatchOptions(ctypes.Structure):
    _fields_ = [("graph_steps", ctypes.c_int), ("autotune", ctypes.c_int),
                ("tile_height", ctypes.c_int), ("blocks_per_sm", ctypes.c_int)]


class BatchInfo(ctypes.Structure):
    _fields_ = [("instances", ctypes.c_int), ("cells", ctypes.c_int64),
                ("steps_done", ctypes.c_int64), ("tile_height", ctypes.c_int),
                ("grid_blocks", ctypes.c_int), ("graph_steps", ctypes.c_int),
                ("tuned_candidates", ctypes.c_int), ("tuned_step_ms", ctypes.c_double),
                ("bytes_per_cell_step", ctypes.c_double)]


class AdjointSpec(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int32), ("checkpoint_every", ctypes.c_int32),
                ("window_begin", ctypes.c_int32), ("window_end", ctypes.c_int32),
                ("objective", ctypes.c_int32)]


class AdjointResult(ctypes.Structure):
    _fields_ = [("J", ctypes.c_double), ("dJ_du_in", ctypes.c_double),
                ("dJ_dtau", ctypes.c_double), ("seconds_forward", ctypes.c_double),
                ("seconds_reverse", ctypes.c_double), ("device_bytes", ctypes.c_int64)]


# Every exported entry point with its ctypes signature (argtypes, restype).
SIGNATURES = {
    "cflbm_config_default": ([ctypes.POINTER(Config)], ctypes.c_int),
    "cflbm_create": ([ctypes.POINTER(Config), ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "cflbm_destroy": ([ctypes.c_void_p], ctypes.c_int),
    "cflbm_step": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "cflbm_synchronize": ([ctypes.c_void_p], ctypes.c_int),
    "cflbm_selftest_wait_timeout": ([ctypes.c_void_p, ctypes.c_int64], ctypes.c_int),
    "cflbm_macros": ([ctypes.c_void_p, _dp, _dp, _dp, _dp], ctypes.c_int),
    "cflbm_macros_device": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                             ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "cflbm_forces": ([ctypes.c_void_p, _dp, _dp], ctypes.c_int),
    "cflbm_forces_async": ([ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "cflbm_force_history": ([ctypes.c_void_p, _dp, ctypes.c_int64,
                             ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
    "cflbm_mass": ([ctypes.c_void_p, _dp, _dp], ctypes.c_int),
    "cflbm_get_f": ([ctypes.c_void_p, _dp], ctypes.c_int),
    "cflbm_get_f_stream": ([ctypes.c_void_p, _dp], ctypes.c_int),
    "cflbm_get_solid": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint8)], ctypes.c_int),
    "cflbm_set_f": ([ctypes.c_void_p, _dp, ctypes.c_int64], ctypes.c_int),
    "cflbm_get_info": ([ctypes.c_void_p, ctypes.POINTER(Info)], ctypes.c_int),
    "cflbm_write_tecplot": ([ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int], ctypes.c_int),
    "cflbm_write_tecplot_fields": ([ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, _dp, _dp, _dp, _dp, ctypes.c_int],
                                   ctypes.c_int),
    "cflbm_get_stream": ([ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "cflbm_set_timing": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "cflbm_get_timing": ([ctypes.c_void_p, _dp, ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
    "cflbm_domain_sums_noalloc": ([ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    "cflbm_batch_options_default": ([ctypes.POINTER(BatchOptions)], ctypes.c_int),
    "cflbm_batch_create": ([ctypes.POINTER(Config), ctypes.c_int, ctypes.POINTER(BatchOptions),
                            ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int),
    "cflbm_batch_destroy": ([ctypes.c_void_p], ctypes.c_int),
    "cflbm_batch_step": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int),
    "cflbm_batch_synchronize": ([ctypes.c_void_p], ctypes.c_int),
    "cflbm_batch_handle": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_void_p),
    "cflbm_batch_get_info": ([ctypes.c_void_p, ctypes.POINTER(BatchInfo)], ctypes.c_int),
    "cflbm_adjoint": ([ctypes.c_void_p, ctypes.POINTER(AdjointSpec), _dp,
                       ctypes.POINTER(AdjointResult)], ctypes.c_int),
    "cflbm_last_error": ([], ctypes.c_char_p),
    "cflbm_launch_count": ([], ctypes.c_int64),
}


class CflbmError(RuntimeError):
    def __init__(self, code: int, fn: str, msg: str):
        super().__init__(f"{fn} failed ({ERRORS.get(code, code)}): {msg}")
        self.code = code


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; "
            "g.build()'` (the solver has no CPU fallback)")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    return lib


lib = _load()


def check(rc: int, fn: str) -> None:
    if rc != 0:
        msg = lib.cflbm_last_error()
        raise CflbmError(rc, fn, msg.decode() if msg else "")
