"""Python front end of the GPU solver (thin: every call goes to libcflbm.so)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib as C


def _ptr(a, t=ctypes.c_double):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(t))


class Solver:
    """One channel (or reference-profile box) resident on one GPU.

    Keyword arguments are the fields of ``cflbm_config`` (include/cflbm.h);
    ``solid`` (uint8, shape (nz, ny, nx) or (ny, nx)), ``alpha`` (float64, same
    shape) and ``ref_ran`` (int32 over the reference's ghosted box) are numpy
    arrays.  ``storage``/``compute``/``profile``/``wall_*``/``geom`` accept the
    integer constants or the names "fp64", "fp32", "fp16dev", "channel",
    "ref2d", "ref3d", "ref2ds", "freeslip", "noslip", "periodic", "cylinder", "sphere".
    """

    _names = {
        "storage": {"fp64": C.STORE_FP64, "fp32": C.STORE_FP32, "fp16dev": C.STORE_FP16DEV},
        "compute": {"fp64": C.COMPUTE_FP64, "fp32": C.COMPUTE_FP32, "df64": C.COMPUTE_DF64},
        "profile": {"channel": C.PROFILE_CHANNEL, "ref2d": C.PROFILE_REF2D,
                    "ref2ds": C.PROFILE_REF2DS,
                    "ref3d": C.PROFILE_REF3D},
        "wall_y": {"freeslip": C.WALL_FREESLIP, "noslip": C.WALL_NOSLIP,
                   "periodic": C.WALL_PERIODIC},
        "wall_z": {"freeslip": C.WALL_FREESLIP, "noslip": C.WALL_NOSLIP,
                   "periodic": C.WALL_PERIODIC},
        "geom": {"none": C.GEOM_NONE, "cylinder": C.GEOM_CYLINDER, "sphere": C.GEOM_SPHERE},
        "layout": {"soa": C.LAYOUT_SOA, "rows": C.LAYOUT_ROWS},
        "rounding": {"nearest": C.ROUND_NEAREST, "stochastic": C.ROUND_STOCHASTIC},
    }

    def __init__(self, **kw):
        cfg, keep = make_config(**kw)
        h = ctypes.c_void_p()
        C.check(C.lib.cflbm_create(ctypes.byref(cfg), ctypes.byref(h)), "cflbm_create")
        self._init_from(h, cfg, owned=True)

    @classmethod
    def _wrap(cls, h, cfg):
        """A view of a handle owned elsewhere (a batch instance)."""
        obj = cls.__new__(cls)
        obj._init_from(ctypes.c_void_p(h), cfg, owned=False)
        return obj

    def _init_from(self, h, cfg, owned):
        self._h = h
        self._owned = owned
        self.cfg = cfg
        self.Q = cfg.lattice
        self.nx, self.ny, self.nz = cfg.nx, cfg.ny, cfg.nz
        self.shape = (self.nz, self.ny, self.nx)

    # -- life cycle ---------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            if getattr(self, "_owned", True):
                C.lib.cflbm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- stepping -----------------------------------------------------------------
    def step(self, n: int = 1):
        C.check(C.lib.cflbm_step(self._h, int(n)), "cflbm_step")
        return self

    def synchronize(self):
        C.check(C.lib.cflbm_synchronize(self._h), "cflbm_synchronize")

    # -- results ------------------------------------------------------------------
    def macros(self):
        """(u, v, w, p) of the last step, each shaped (nz, ny, nx)."""
        out = [np.empty(self.shape) for _ in range(4)]
        C.check(C.lib.cflbm_macros(self._h, *[_ptr(a) for a in out]), "cflbm_macros")
        return tuple(out)

    def macros_device(self, u, v, w, p):
        """Copy the macroscopic fields into device buffers (e.g. torch tensors)."""
        ptrs = [None if t is None else ctypes.c_void_p(t.data_ptr()) for t in (u, v, w, p)]
        C.check(C.lib.cflbm_macros_device(self._h, *ptrs), "cflbm_macros_device")

    def forces(self):
        f = np.zeros(3)
        c = np.zeros(2)
        C.check(C.lib.cflbm_forces(self._h, _ptr(f), _ptr(c)), "cflbm_forces")
        return f, c

    def forces_async(self, ptr: int):
        """Queue a copy of the last step's (Fx, Fy, Fz) to host address `ptr`
        (3 doubles, page-locked for the copy to be asynchronous); valid after
        synchronize()."""
        C.check(C.lib.cflbm_forces_async(self._h, ctypes.c_void_p(int(ptr))),
                "cflbm_forces_async")

    def force_history(self, max_steps: int | None = None):
        if max_steps is None:
            max_steps = self.info().steps_done
        out = np.zeros((max(int(max_steps), 1), 3))
        n = ctypes.c_int64()
        C.check(C.lib.cflbm_force_history(self._h, _ptr(out), int(max_steps), ctypes.byref(n)),
                "cflbm_force_history")
        return out[: n.value]

    def adjoint(self, steps: int, checkpoint_every: int, window: tuple[int, int],
                objective: str = "drag"):
        """cflbm_adjoint on this (fresh) handle: runs `steps` forward steps and the
        reverse sweep.  Returns J, dJ/dalpha (shape (ny, nx)), dJ/du_in,
        dJ/dtau and the timings."""
        spec = C.AdjointSpec(int(steps), int(checkpoint_every), int(window[0]), int(window[1]),
                             {"drag": 0, "lift": 1}[objective])
        res = C.AdjointResult()
        g = np.zeros((self.ny, self.nx))
        C.check(C.lib.cflbm_adjoint(self._h, ctypes.byref(spec), _ptr(g), ctypes.byref(res)),
                "cflbm_adjoint")
        return {"J": res.J, "dJ_dalpha": g, "dJ_du_in": res.dJ_du_in, "dJ_dtau": res.dJ_dtau,
                "seconds_forward": res.seconds_forward, "seconds_reverse": res.seconds_reverse,
                "device_bytes": res.device_bytes}

    def mass(self):
        m = np.zeros(1)
        mom = np.zeros(3)
        C.check(C.lib.cflbm_mass(self._h, _ptr(m), _ptr(mom)), "cflbm_mass")
        return float(m[0]), mom

    def get_f(self):
        out = np.empty((self.Q,) + self.shape)
        C.check(C.lib.cflbm_get_f(self._h, _ptr(out)), "cflbm_get_f")
        return out

    def get_f_stream(self):
        """Post-stream (pre-collision) populations of the last step, shaped
        (Q, nz, ny, nx): what the reference's f holds after Update."""
        out = np.empty((self.Q,) + self.shape)
        C.check(C.lib.cflbm_get_f_stream(self._h, _ptr(out)), "cflbm_get_f_stream")
        return out

    def solid(self):
        """Interior solid mask (1 = solid), shaped (nz, ny, nx)."""
        out = np.empty(self.shape, np.uint8)
        C.check(C.lib.cflbm_get_solid(self._h, _ptr(out, ctypes.c_uint8)), "cflbm_get_solid")
        return out

    def set_f(self, f, steps_done: int = 0):
        a = np.ascontiguousarray(f, np.float64).reshape((self.Q,) + self.shape)
        C.check(C.lib.cflbm_set_f(self._h, _ptr(a), int(steps_done)), "cflbm_set_f")

    def info(self) -> C.Info:
        i = C.Info()
        C.check(C.lib.cflbm_get_info(self._h, ctypes.byref(i)), "cflbm_get_info")
        return i

    def stream_ptr(self) -> int:
        """cudaStream_t of the handle (e.g. for torch.cuda.ExternalStream)."""
        p = ctypes.c_void_p()
        C.check(C.lib.cflbm_get_stream(self._h, ctypes.byref(p)), "cflbm_get_stream")
        return int(p.value or 0)

    def set_timing(self, on: bool = True):
        C.check(C.lib.cflbm_set_timing(self._h, 1 if on else 0), "cflbm_set_timing")

    def timing(self):
        """(sweep_ms_total, boundary_ms_total, n_sweeps, n_boundary) since last call."""
        ms = np.zeros(2)
        n = (ctypes.c_int64 * 2)()
        C.check(C.lib.cflbm_get_timing(self._h, _ptr(ms), n), "cflbm_get_timing")
        return float(ms[0]), float(ms[1]), int(n[0]), int(n[1])

    def write_tecplot(self, path: str, n: int):
        C.check(C.lib.cflbm_write_tecplot(self._h, path.encode(), int(n)), "cflbm_write_tecplot")


def launch_count() -> int:
    return int(C.lib.cflbm_launch_count())


def write_tecplot_fields(path: str, u, v, w, p, n: int) -> None:
    """Write host fields (shape (nz, ny, nx) or (ny, nx)) as the reference's
    Tecplot file; 2-D when the arrays are 2-D or nz == 1 and w is None."""
    u = np.ascontiguousarray(u, np.float64)
    dim = 2 if (u.ndim == 2 or w is None) else 3
    shp = u.shape if u.ndim == 3 else (1,) + u.shape
    arrs = [np.ascontiguousarray(a, np.float64) if a is not None else np.zeros(shp)
            for a in (u, v, w, p)]
    C.check(C.lib.cflbm_write_tecplot_fields(path.encode(), dim, shp[2], shp[1], shp[0],
                                             *[_ptr(a) for a in arrs], int(n)),
            "cflbm_write_tecplot_fields")


_NAMES = Solver._names


def make_config(**kw):
    """A cflbm_config from keyword arguments (see Solver); returns (cfg, buffers
    that must stay alive until the handle is created)."""
    cfg = C.Config()
    C.check(C.lib.cflbm_config_default(ctypes.byref(cfg)), "cflbm_config_default")
    keep = []
    for k, v in kw.items():
        if k in ("solid", "alpha", "ref_ran"):
            if v is None:
                continue
            dt = {"solid": np.uint8, "alpha": np.float64, "ref_ran": np.int32}[k]
            a = np.ascontiguousarray(v, dt)
            keep.append(a)
            t = {"solid": ctypes.c_uint8, "alpha": ctypes.c_double, "ref_ran": ctypes.c_int32}[k]
            setattr(cfg, k, _ptr(a, t))
        elif k in _NAMES and isinstance(v, str):
            setattr(cfg, k, _NAMES[k][v.lower()])
        else:
            setattr(cfg, k, v)
    if cfg.lattice == C.D2Q9:
        cfg.nz = 1
    return cfg, keep


class Batch:
    """Many channel instances advanced together (cflbm_batch_*).

    `configs` is a list of keyword dicts as for Solver (CHANNEL profile, one
    lattice and storage, FP32 arithmetic).  `instance(k)` returns a Solver view of
    instance k for results (macros, forces, force_history, get_f, mass)."""

    def __init__(self, configs, graph_steps=100, autotune=True, tile_height=4,
                 blocks_per_sm=8):
        cfgs = (C.Config * len(configs))()
        keep = []
        for k, kw in enumerate(configs):
            kw = dict(kw)
            kw.setdefault("compute", "fp32")
            c, kp = make_config(**kw)
            keep.extend(kp)
            cfgs[k] = c
        opt = C.BatchOptions()
        C.check(C.lib.cflbm_batch_options_default(ctypes.byref(opt)), "cflbm_batch_options_default")
        opt.graph_steps = graph_steps
        opt.autotune = 1 if autotune else 0
        opt.tile_height = tile_height
        opt.blocks_per_sm = blocks_per_sm
        b = ctypes.c_void_p()
        C.check(C.lib.cflbm_batch_create(cfgs, len(configs), ctypes.byref(opt), ctypes.byref(b)),
                "cflbm_batch_create")
        self._b = b
        self._cfgs = [cfgs[k] for k in range(len(configs))]
        self.n = len(configs)

    def step(self, n=1):
        C.check(C.lib.cflbm_batch_step(self._b, int(n)), "cflbm_batch_step")
        return self

    def synchronize(self):
        C.check(C.lib.cflbm_batch_synchronize(self._b), "cflbm_batch_synchronize")

    def instance(self, k) -> Solver:
        h = C.lib.cflbm_batch_handle(self._b, int(k))
        if not h:
            raise IndexError(k)
        return Solver._wrap(h, self._cfgs[k])

    def info(self) -> C.BatchInfo:
        i = C.BatchInfo()
        C.check(C.lib.cflbm_batch_get_info(self._b, ctypes.byref(i)), "cflbm_batch_get_info")
        return i

    def close(self):
        if getattr(self, "_b", None):
            C.lib.cflbm_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
