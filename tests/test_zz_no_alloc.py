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


def _h_scale(lattice):
    """The per-direction power of two of the FP16 deviation format (f_i times
    it, stored as binary16): 2 / 8 / 32 for D2Q9's rest / axis / diagonal
    directions, 4 / 16 / 64 / 256 for D3Q27's four weight classes."""
    if lattice == 9:
        return np.array([2.0] + [8.0] * 4 + [32.0] * 4)
    return np.array([4.0] + [16.0] * 6 + [64.0] * 12 + [256.0] * 8)


def _encode(f, lattice, storage):
    """Dense [i][z][y][x] populations in a storage format, and their FP64
    values as the GPU decodes them (exact conversions)."""
    if storage == C.STORE_FP64:
        return f, f
    if storage == C.STORE_FP32:
        e = f.astype(np.float32)
        return e, e.astype(np.float64)
    sc = _h_scale(lattice).reshape(-1, 1, 1, 1)
    e = (f * sc).astype(np.float16)
    return e, e.astype(np.float64) / sc


def _host_sums(f64, lattice, solid):
    """Mass (sum of 1 + sum_i f_i) and momentum over fluid cells, in FP64."""
    e = np.array(_E[lattice], np.float64)
    fluid = np.ones(f64.shape[1:], bool) if solid is None else solid == 0
    ff = f64[:, fluid]
    return np.array([np.sum(1.0 + ff.sum(axis=0)), *(e.T @ ff.sum(axis=1))])


_E = {9: [(0, 0, 0), (1, 0, 0), (0, 1, 0), (-1, 0, 0), (0, -1, 0), (1, 1, 0), (-1, 1, 0),
          (-1, -1, 0), (1, -1, 0)],
      27: [(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1),
           (1, 1, 0), (-1, -1, 0), (1, -1, 0), (-1, 1, 0), (1, 0, 1), (-1, 0, -1), (1, 0, -1),
           (-1, 0, 1), (0, 1, 1), (0, -1, -1), (0, 1, -1), (0, -1, 1), (1, 1, 1), (-1, -1, -1),
           (1, -1, 1), (-1, 1, -1), (1, 1, -1), (-1, -1, 1), (1, -1, -1), (-1, 1, 1)]}


def _call(cuda, lattice, storage, case, d_f, d_solid):
    import torch
    stream = torch.cuda.current_stream(cuda)
    d_out = torch.full((4,), float("nan"), dtype=torch.float64, device=cuda)
    rc = C.lib.cflbm_domain_sums_noalloc(
        lattice, storage, case["nx"], case["ny"], case["nz"],
        ctypes.c_void_p(d_f.data_ptr()),
        None if d_solid is None else ctypes.c_void_p(d_solid.data_ptr()),
        ctypes.c_void_p(d_out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    C.check(rc, "cflbm_domain_sums_noalloc")
    torch.cuda.synchronize()
    return d_out.cpu().numpy()


def _close(got, ref):
    assert np.all(np.isfinite(got))
    assert abs(got[0] - ref[0]) <= REL_TOL * abs(ref[0])
    scale = max(np.max(np.abs(ref[1:])), 1e-300)
    assert np.max(np.abs(got[1:] - ref[1:])) <= 1e-10 * scale


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
    for _ in range(2):
        _close(_call(cuda, lattice, C.STORE_FP64, case, d_f, d_solid), ref)


@pytest.mark.parametrize("storage", [C.STORE_FP32, C.STORE_FP16DEV])
@pytest.mark.parametrize("lattice", [9, 27])
def test_noalloc_sums_every_storage_twice(cuda, lattice, storage):
    """FP32 and FP16-deviation arrays (the handle's own state after 25 steps,
    encoded on the host) against FP64 sums of the same decoded values, with the
    solid mask and without it (every cell counted), each twice in a row."""
    import torch
    case = _case(lattice)
    with Solver(**case) as s:
        s.step(25)
        f = s.get_f()
    enc, dec = _encode(f, lattice, storage)
    solid = _solid(case)
    d_f = torch.from_numpy(np.ascontiguousarray(enc)).to(cuda)
    d_solid = torch.from_numpy(solid).to(cuda)
    for mask in (solid, None):
        ref = _host_sums(dec, lattice, mask)
        for _ in range(2):
            _close(_call(cuda, lattice, storage, case, d_f, None if mask is None else d_solid),
                   ref)


def test_noalloc_rejects_oversized_grid(cuda):
    rc = C.lib.cflbm_domain_sums_noalloc(27, C.STORE_FP64, 1024, 1024, 1024, ctypes.c_void_p(16),
                                         None, ctypes.c_void_p(16), None)
    assert rc == 1
    assert b"exceeds" in C.lib.cflbm_last_error()
