"""The allocation-free domain-sum entry point (cflbm_domain_sums_noalloc).

Some callers cannot call cudaMalloc -- a memory pool or framework that owns all
device memory, or a fixed memory budget -- yet hold populations on the device
and want the FP64 mass/momentum check.  This entry point serves them with a
static device scratch array instead of allocating.  The test calls it through
the C ABI on a handle's state and checks it against the handle-based
cflbm_mass(), twice in a row (the second call reuses the static scratch the
first one left behind).  This file is named to be collected last.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from cflbm import Solver
from cflbm import _lib as C

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12  # FP64 sums in a different order than cflbm_mass


def _case(lattice):
    if lattice == 9:
        return dict(lattice=9, nx=160, ny=41, nz=1, tau0=0.03, u0=0.05, wall_y="freeslip",
                    geom="cylinder", cx=32, cy=20, diam=10, perturb_amp=1e-3, seed=1234)
    return dict(lattice=27, nx=64, ny=32, nz=12, tau0=0.0192, u0=0.04, wall_y="freeslip",
                wall_z="periodic", geom="cylinder", cx=16, cy=16, diam=8, perturb_amp=1e-3,
                seed=1234)


def _solid(case):
    nz = case["nz"]
    yy, xx = np.mgrid[0:case["ny"], 0:case["nx"]]
    disk = (xx - case["cx"]) ** 2 + (yy - case["cy"]) ** 2 <= 0.25 * case["diam"] ** 2
    return np.repeat(disk[None].astype(np.uint8), nz, axis=0)


@pytest.mark.parametrize("lattice", [9, 27])
def test_noalloc_sums_match_cflbm_mass_twice(cuda, lattice):
    import torch
    case = _case(lattice)
    with Solver(**case) as s:
        s.step(25)
        f = s.get_f()
        mass, mom = s.mass()
        ref = np.array([mass, *mom])
    d_f = torch.from_numpy(np.ascontiguousarray(f)).to(cuda)
    d_solid = torch.from_numpy(_solid(case)).to(cuda)
    stream = torch.cuda.current_stream(cuda)
    for _ in range(2):
        d_out = torch.full((4,), float("nan"), dtype=torch.float64, device=cuda)
        rc = C.lib.cflbm_domain_sums_noalloc(
            lattice, C.STORE_FP64, case["nx"], case["ny"], case["nz"],
            ctypes.c_void_p(d_f.data_ptr()), ctypes.c_void_p(d_solid.data_ptr()),
            ctypes.c_void_p(d_out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
        C.check(rc, "cflbm_domain_sums_noalloc")
        torch.cuda.synchronize()
        got = d_out.cpu().numpy()
        assert np.all(np.isfinite(got))
        assert abs(got[0] - ref[0]) <= REL_TOL * abs(ref[0])
        scale = max(np.max(np.abs(ref[1:])), 1e-300)
        assert np.max(np.abs(got[1:] - ref[1:])) <= 1e-10 * scale


def test_noalloc_rejects_oversized_grid(cuda):
    rc = C.lib.cflbm_domain_sums_noalloc(27, C.STORE_FP64, 1024, 1024, 1024, ctypes.c_void_p(16),
                                         None, ctypes.c_void_p(16), None)
    assert rc == 1
    assert b"exceeds" in C.lib.cflbm_last_error()
