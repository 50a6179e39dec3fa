"""cflbm: GB300-native lattice-Boltzmann cylinder/sphere channel-flow solver.

The compute path is libcflbm.so (hand-written CUDA for sm_103a behind the C ABI
of include/cflbm.h); this package is a thin ctypes front end plus
post-processing.  Importing it loads the library and raises if it is missing.
"""
from . import _lib  # noqa: F401  (loads libcflbm.so, fails loudly if absent)
from ._lib import (COMPUTE_FP32, COMPUTE_FP64, D2Q9, D3Q27, GEOM_CYLINDER, GEOM_NONE,  # noqa
                   GEOM_SPHERE, PROFILE_CHANNEL, PROFILE_REF2D, PROFILE_REF2DS, PROFILE_REF3D,
                   STORE_FP16DEV,
                   STORE_FP32, STORE_FP64, WALL_FREESLIP, WALL_NOSLIP, WALL_PERIODIC, CflbmError)
from .solver import Batch, Solver, launch_count  # noqa: F401
from . import analysis  # noqa: F401

__all__ = ["Batch", "Solver", "CflbmError", "analysis", "launch_count"]
