"""Oracle parity at the benchmark problems' own grid sizes.

* The D3Q27 spanwise-cylinder problem at its full 512x128x128 grid (D = 32 at
  (128, 64), free-slip y, periodic z, u_in = 0.04, Re = 200): a few steps of
  every arithmetic and storage form against the FP64 oracle's run of the same
  steps -- u, v, w, p, the post-collision populations and the per-step force.
* The precision problem's 768x384x384 sphere grid (D = 64 at (192, 192, 192),
  free-slip faces, u_in = 0.03, Re = 300): more than 2^31 population elements
  per buffer, so every 64-bit index path runs; two steps against the oracle
  (about 55 GB of host memory and a minute per step on the host's cores).

Tolerances (relative L-inf, scaled by the field's max |value|) as in
test_gpu_parity.py: FP64 arithmetic 1e-10 (fields) / 1e-9 (force); double-float
1e-9; FP32 collision 2e-5; FP16-deviation storage 3e-3, its velocity
components scaled by the flow speed max |u| (v and w are near zero over most
of these grids, so binary16's absolute resolution is what they see)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_err
from oracle import oracle as O

from cflbm import Solver

pytestmark = pytest.mark.gpu

STEPS2 = 4
CYL = dict(lattice=27, nx=512, ny=128, nz=128, tau0=3 * 0.04 * 32 / 200, u0=0.04,
           wall_y="freeslip", wall_z="periodic", geom="cylinder", cx=128.0, cy=64.0, diam=32.0,
           perturb_amp=1e-3, seed=1234)
FORMS = [("fp64", "fp64", 1e-10, 1e-9), ("fp64", "df64", 1e-9, 1e-9),
         ("fp64", "fp32", 2e-5, 2e-5), ("fp32", "fp32", 2e-5, 2e-5),
         ("fp16dev", "fp32", 3e-3, 3e-3)]


@pytest.fixture(scope="module")
def cyl_oracle():
    cfg = O.channel_cfg(27, 512, 128, 128, tau0=CYL["tau0"], u_in=0.04, wall_y=O.WALL_FREESLIP,
                        wall_z=O.WALL_PERIODIC, geom=O.GEOM_CYLINDER, cx=128.0, cy=64.0,
                        diam=32.0, amp=1e-3, seed=1234)
    return O.channel(cfg, STEPS2)


@pytest.mark.parametrize("storage,compute,tol,ftol", FORMS)
def test_cylinder_512x128x128_matches_oracle(cuda, cyl_oracle, storage, compute, tol, ftol):
    o = cyl_oracle
    with Solver(storage=storage, compute=compute, force_history=16, **CYL) as s:
        s.step(STEPS2)
        u, v, w, p = s.macros()
        fh = s.force_history()
        fpost = s.get_f()
    speed = float(np.max(np.abs(o["u"])))
    for k, a in (("u", u), ("v", v), ("w", w), ("p", p)):
        err = rel_err(a, o[k])
        if storage == "fp16dev" and k != "p":
            err = float(np.max(np.abs(a - o[k]))) / speed
        assert err < tol, (k, err)
    assert rel_err(fpost, o["fpost"]) < tol
    assert rel_err(fh, o["force"]) < ftol


SPHERE = dict(lattice=27, nx=768, ny=384, nz=384, tau0=3 * 0.03 * 64 / 300, u0=0.03,
              wall_y="freeslip", wall_z="freeslip", geom="sphere", cx=192.0, cy=192.0, cz=192.0,
              diam=64.0, perturb_amp=1e-3, seed=1234)
STEPS3 = 2


@pytest.fixture(scope="module")
def sphere_oracle():
    cfg = O.channel_cfg(27, 768, 384, 384, tau0=SPHERE["tau0"], u_in=0.03,
                        wall_y=O.WALL_FREESLIP, wall_z=O.WALL_FREESLIP, geom=O.GEOM_SPHERE,
                        cx=192.0, cy=192.0, cz=192.0, diam=64.0, amp=1e-3, seed=1234)
    return O.channel(cfg, STEPS3, want_f=False)


@pytest.mark.parametrize("storage,compute,tol,ftol", FORMS[:3])
def test_sphere_768x384x384_matches_oracle(cuda, sphere_oracle, storage, compute, tol, ftol):
    o = sphere_oracle
    with Solver(storage=storage, compute=compute, force_history=16, **SPHERE) as s:
        info = s.info()
        assert 27 * info.pitch_x * (384 + 2) * (384 + 2) > 2 ** 31  # elements per buffer
        s.step(STEPS3)
        u, v, w, p = s.macros()
        fh = s.force_history()
    for k, a in (("u", u), ("v", v), ("w", w), ("p", p)):
        assert rel_err(a, o[k]) < tol, (k, rel_err(a, o[k]))
    assert rel_err(fh, o["force"]) < ftol
