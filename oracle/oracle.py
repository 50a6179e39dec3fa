"""ctypes front end of the CPU oracle: TEST INFRASTRUCTURE ONLY.

Imported by tests/, by ``__graft_entry__.smoke()`` and by bench.py's CPU
baseline leg, never by the product package.  Wraps oracle/liboracle.so
(oracle/lbm_oracle.cpp) and runs the compiled reference binaries in
oracle/_ref/ when they exist.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile

import numpy as np

from . import build as _build  # type: ignore

WALL_FREESLIP, WALL_NOSLIP, WALL_PERIODIC = 0, 1, 2
GEOM_NONE, GEOM_CYLINDER, GEOM_SPHERE = 0, 1, 2

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


class ChannelCfg(ctypes.Structure):
    _fields_ = [
        ("Q", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("tau0", ctypes.c_double), ("u_in", ctypes.c_double),
        ("wall_y", ctypes.c_int), ("wall_z", ctypes.c_int), ("geom", ctypes.c_int),
        ("cx", ctypes.c_double), ("cy", ctypes.c_double), ("cz", ctypes.c_double),
        ("diam", ctypes.c_double), ("amp", ctypes.c_double), ("seed", ctypes.c_uint64),
        ("alpha", _dp), ("solid", ctypes.POINTER(ctypes.c_uint8)),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = ctypes.CDLL(path)
        L.oracle_ref2d_run.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                       ctypes.c_double, _ip, ctypes.c_int, _dp, _dp, _dp,
                                       _dp, _dp, _dp, ctypes.c_int]
        L.oracle_ref2ds_run.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                        ctypes.c_double, _ip, ctypes.c_int, _dp, _dp, _dp,
                                        _dp, _dp, ctypes.c_int]
        L.oracle_ref3d_run.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_double, ctypes.c_double, _ip, ctypes.c_int,
                                       _dp, _dp, _dp, _dp, _dp, _dp, ctypes.c_int]
        L.oracle_channel_run.argtypes = [ctypes.POINTER(ChannelCfg), ctypes.c_int, _dp, _dp,
                                         _dp, _dp, _dp, _dp, ctypes.c_int, _dp, _dp]
        L.oracle_channel_mask.argtypes = [ctypes.POINTER(ChannelCfg),
                                          ctypes.POINTER(ctypes.c_uint8)]
        L.oracle_perturbation.argtypes = [ctypes.c_uint64, ctypes.c_long, ctypes.c_double]
        L.oracle_perturbation.restype = ctypes.c_double
        L.oracle_lattice.argtypes = [ctypes.c_int, _ip, _dp, _ip]
        _lib = L
    return _lib


def _p(a, t=_dp):
    return None if a is None else a.ctypes.data_as(t)


def lattice(Q: int):
    e = np.zeros((Q, 3), np.int32)
    t = np.zeros(Q, np.float64)
    bb = np.zeros(Q, np.int32)
    assert lib().oracle_lattice(Q, _p(e, _ip), _p(t), _p(bb, _ip)) == 0
    return e, t, bb


def ref2d(nx, ny, tau0, u0, ran, steps, nthreads=0):
    """Run the 2-D reference restatement; arrays keep the reference's ghost ring."""
    lx, ly = nx + 4, ny + 4
    ran = np.ascontiguousarray(ran, np.int32).reshape(lx, ly)
    out = dict(f=np.zeros((9, lx, ly)), fpost=np.zeros((9, lx, ly)), u=np.zeros((lx, ly)),
               v=np.zeros((lx, ly)), p=np.zeros((lx, ly)), force=np.zeros((max(steps, 1), 2)))
    rc = lib().oracle_ref2d_run(nx, ny, tau0, u0, _p(ran, _ip), steps, _p(out["f"]),
                                _p(out["fpost"]), _p(out["u"]), _p(out["v"]), _p(out["p"]),
                                _p(out["force"]), nthreads)
    assert rc == 0
    out["force"] = out["force"][:steps]
    return out


def ref2ds(nx, ny, tau0, u0, ran, steps, nthreads=0):
    """Run the serial 2-D reference restatement ("Kokkos/lbm.cpp"); nx, ny are the
    interior nodes (the reference's sx + 1, sy + 1); arrays keep its ghost ring."""
    lx, ly = nx + 4, ny + 4
    ran = np.ascontiguousarray(ran, np.int32).reshape(lx, ly)
    out = dict(f=np.zeros((9, lx, ly)), fpost=np.zeros((9, lx, ly)), u=np.zeros((lx, ly)),
               v=np.zeros((lx, ly)), p=np.zeros((lx, ly)))
    rc = lib().oracle_ref2ds_run(nx, ny, tau0, u0, _p(ran, _ip), steps, _p(out["f"]),
                                 _p(out["fpost"]), _p(out["u"]), _p(out["v"]), _p(out["p"]),
                                 nthreads)
    assert rc == 0
    return out


def ref3d(nx, ny, nz, tau0, u0, ran, steps, nthreads=0, want_f=True):
    lx, ly, lz = nx + 6, ny + 6, nz + 6
    ran = np.ascontiguousarray(ran, np.int32).reshape(lx, ly, lz)
    shp = (lx, ly, lz)
    out = dict(u=np.zeros(shp), v=np.zeros(shp), w=np.zeros(shp), p=np.zeros(shp))
    if want_f:
        out["f"] = np.zeros((27,) + shp)
        out["fpost"] = np.zeros((27,) + shp)
    rc = lib().oracle_ref3d_run(nx, ny, nz, tau0, u0, _p(ran, _ip), steps, _p(out.get("f")),
                                _p(out.get("fpost")), _p(out["u"]), _p(out["v"]),
                                _p(out["w"]), _p(out["p"]), nthreads)
    assert rc == 0
    return out


def channel_cfg(Q, nx, ny, nz=1, tau0=0.03, u_in=0.05, wall_y=WALL_FREESLIP,
                wall_z=WALL_PERIODIC, geom=GEOM_CYLINDER, cx=0.0, cy=0.0, cz=0.0, diam=0.0,
                amp=1e-3, seed=1234, alpha=None, solid=None):
    c = ChannelCfg(Q, nx, ny, nz if Q == 27 else 1, tau0, u_in, wall_y, wall_z, geom, cx, cy,
                   cz, diam, amp, seed, None, None)
    keep = []
    if alpha is not None:
        a = np.ascontiguousarray(alpha, np.float64)
        keep.append(a)
        c.alpha = _p(a)
    if solid is not None:
        s = np.ascontiguousarray(solid, np.uint8)
        keep.append(s)
        c.solid = s.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
    c._keep = keep  # keep buffers alive with the struct
    return c


def channel(cfg: ChannelCfg, steps: int, nthreads=0, want_f=True, want_fstream=False):
    """Run the channel-profile oracle.  Arrays are interior only, x fastest;
    ``fpost`` is the post-collision state after the run, ``fstream`` (on
    request) the post-stream state the run ends with (the reference's f after
    Update); ``step_seconds`` holds the wall time of every step
    (initialisation excluded)."""
    nz = cfg.nz if cfg.Q == 27 else 1
    shp = (nz, cfg.ny, cfg.nx)
    out = dict(u=np.zeros(shp), v=np.zeros(shp), w=np.zeros(shp), p=np.zeros(shp),
               force=np.zeros((max(steps, 1), 3)), step_seconds=np.zeros(max(steps, 1)))
    if want_f:
        out["fpost"] = np.zeros((cfg.Q,) + shp)
    if want_fstream:
        out["fstream"] = np.zeros((cfg.Q,) + shp)
    rc = lib().oracle_channel_run(ctypes.byref(cfg), steps, _p(out.get("fpost")),
                                  _p(out["u"]), _p(out["v"]), _p(out["w"]), _p(out["p"]),
                                  _p(out["force"]), nthreads, _p(out["step_seconds"]),
                                  _p(out.get("fstream")))
    assert rc == 0
    out["force"] = out["force"][:steps]
    out["step_seconds"] = out["step_seconds"][:steps]
    return out


def channel_mask(cfg: ChannelCfg):
    nz = cfg.nz if cfg.Q == 27 else 1
    m = np.zeros((nz, cfg.ny, cfg.nx), np.uint8)
    lib().oracle_channel_mask(ctypes.byref(cfg), m.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
    return m


def perturbation(seed, cell, amp):
    return lib().oracle_perturbation(seed, cell, amp)


# ---- the compiled reference (only where oracle/_ref exists) -------------------
def ref_binary(name: str) -> str | None:
    p = os.path.join(os.path.dirname(_build.oracle_lib_path()), "_ref", name)
    return p if os.path.exists(p) else None


def run_ref2d_binary(nx, ny, tau0, u0, steps, outdir=None):
    exe = ref_binary("ref2d")
    if exe is None:
        return None
    outdir = outdir or tempfile.mkdtemp(prefix="ref2d_")
    subprocess.run([exe, outdir, str(nx), str(ny), repr(tau0), repr(u0), str(steps)],
                   check=True, capture_output=True)
    lx, ly = nx + 4, ny + 4
    rd = lambda n, dt=np.float64: np.fromfile(os.path.join(outdir, n), dt)  # noqa: E731
    return dict(dir=outdir, ran=rd("ran.i32", np.int32).reshape(lx, ly),
                f=rd("f.f64").reshape(9, lx, ly), fpost=rd("fpost.f64").reshape(9, lx, ly),
                u=rd("u.f64").reshape(lx, ly), v=rd("v.f64").reshape(lx, ly),
                p=rd("p.f64").reshape(lx, ly))


def run_ref2ds_binary(sx, sy, tau0, u0, steps, outdir=None):
    """The compiled serial 2-D reference ("Kokkos/"); its interior is (sx + 1) x
    (sy + 1) nodes."""
    exe = ref_binary("ref2ds")
    if exe is None:
        return None
    outdir = outdir or tempfile.mkdtemp(prefix="ref2ds_")
    subprocess.run([exe, outdir, str(sx), str(sy), repr(tau0), repr(u0), str(steps)],
                   check=True, capture_output=True)
    lx, ly = sx + 5, sy + 5
    rd = lambda n, dt=np.float64: np.fromfile(os.path.join(outdir, n), dt)  # noqa: E731
    return dict(dir=outdir, ran=rd("ran.i32", np.int32).reshape(lx, ly),
                f=rd("f.f64").reshape(9, lx, ly), fpost=rd("fpost.f64").reshape(9, lx, ly),
                u=rd("u.f64").reshape(lx, ly), v=rd("v.f64").reshape(lx, ly),
                p=rd("p.f64").reshape(lx, ly))


def run_ref3d_binary(nx, ny, nz, tau0, u0, steps, outdir=None):
    exe = ref_binary("ref3d")
    if exe is None:
        return None
    outdir = outdir or tempfile.mkdtemp(prefix="ref3d_")
    subprocess.run([exe, "run", outdir, str(nx), str(ny), str(nz), repr(tau0), repr(u0),
                    str(steps)], check=True, capture_output=True)
    s = (nx + 6, ny + 6, nz + 6)
    rd = lambda n, dt=np.float64: np.fromfile(os.path.join(outdir, n), dt)  # noqa: E731
    return dict(dir=outdir, ran=rd("ran.i32", np.int32).reshape(s),
                f=rd("f.f64").reshape((27,) + s), fpost=rd("fpost.f64").reshape((27,) + s),
                u=rd("u.f64").reshape(s), v=rd("v.f64").reshape(s), w=rd("w.f64").reshape(s),
                p=rd("p.f64").reshape(s))
