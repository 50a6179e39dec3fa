"""C ABI library: loads, exports every declared entry point, validates input,
and writes the reference's Tecplot bytes (all without a GPU)."""
from __future__ import annotations

import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, load_golden

import cflbm
from cflbm import _lib as C
from cflbm.solver import write_tecplot_fields


def declared_symbols():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            names |= set(re.findall(r"^\s*(?:const\s+)?[A-Za-z_0-9]+\s*\**\s*(cflbm_\w+)\s*\(",
                                    txt, re.M))
    return names


def test_library_exports_every_declared_symbol():
    names = declared_symbols()
    assert len(names) >= 17
    out = subprocess.run(["nm", "-D", "--defined-only", C.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\sT\s(cflbm_\w+)", out))
    missing = names - exported
    assert not missing, missing
    for n in names:
        assert hasattr(C.lib, n)
    # every declared symbol has a ctypes signature in the binding
    assert names <= set(C.SIGNATURES)


def test_struct_layouts_match_the_header(tmp_path):
    """Every struct of include/cflbm.h has the size and field offsets the
    ctypes binding assumes (compiled with the host C compiler)."""
    structs = {"cflbm_config": C.Config, "cflbm_info": C.Info,
               "cflbm_batch_options": C.BatchOptions, "cflbm_batch_info": C.BatchInfo,
               "cflbm_adjoint_spec": C.AdjointSpec, "cflbm_adjoint_result": C.AdjointResult}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "cflbm.h"',
             'int main(void) {']
    for cname, py in structs.items():
        lines.append(f'  printf("{cname} %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'  printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    lines += ['  return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe)], check=True)
    got = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True,
                                                 check=True).stdout.splitlines())
    for cname, py in structs.items():
        assert int(got[cname]) == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(got[f"{cname}.{f}"]) == getattr(py, f).offset, (cname, f)


def test_smooth_porosity_field():
    from cflbm.adjoint import smooth_porosity
    a = smooth_porosity(64, 40, (10, 5, 42, 37), seed=3)
    b = smooth_porosity(64, 40, (10, 5, 42, 37), seed=3)
    assert np.array_equal(a, b)
    assert a.max() == 1.0 and a.min() >= 0.0
    assert np.all(a[:5] == 0) and np.all(a[37:] == 0) and np.all(a[:, :10] == 0)
    assert np.all(a[5:37, 10:42] > 0)


def test_build_targets_sm103a_only():
    from cflbm import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_config_default():
    cfg = C.Config()
    assert C.lib.cflbm_config_default(ctypes.byref(cfg)) == 0
    assert cfg.lattice == 9 and cfg.nx == 64 and cfg.ny == 32
    assert cfg.storage == C.STORE_FP64 and cfg.compute == C.COMPUTE_FP64
    assert cfg.tau0 == 0.03 and cfg.u0 == 0.05
    assert cfg.layout == C.LAYOUT_ROWS and cfg.rounding == C.ROUND_STOCHASTIC


@pytest.mark.parametrize("field,value", [("lattice", 7), ("nx", 2), ("storage", 9),
                                         ("compute", 5), ("profile", 4), ("wall_y", 3),
                                         ("tau0", -0.6), ("force_history", -1),
                                         ("layout", 2), ("rounding", 2)])
def test_create_rejects_bad_config_before_touching_the_gpu(field, value):
    cfg = C.Config()
    C.lib.cflbm_config_default(ctypes.byref(cfg))
    setattr(cfg, field, value)
    h = ctypes.c_void_p()
    rc = C.lib.cflbm_create(ctypes.byref(cfg), ctypes.byref(h))
    assert rc == 1
    assert not h.value
    assert C.lib.cflbm_last_error()


def test_profile_lattice_mismatch_rejected():
    cfg = C.Config()
    C.lib.cflbm_config_default(ctypes.byref(cfg))
    cfg.profile = C.PROFILE_REF3D
    h = ctypes.c_void_p()
    assert C.lib.cflbm_create(ctypes.byref(cfg), ctypes.byref(h)) == 1
    assert b"REF3D" in C.lib.cflbm_last_error()


def test_null_handle_calls_fail_cleanly():
    assert C.lib.cflbm_step(None, 1) == 1
    assert C.lib.cflbm_destroy(None) == 0
    with pytest.raises(cflbm.CflbmError):
        C.check(C.lib.cflbm_synchronize(None), "cflbm_synchronize")


def test_tecplot_2d_bytes_match_reference(tmp_path):
    g = load_golden("ref2d_96x40")
    path = str(tmp_path / "out.plt")
    write_tecplot_fields(path, g["u"], g["v"], None, g["p"], 1)
    ref = open(os.path.join(GOLDEN, "ref2d_96x40_output1.plt"), "rb").read()
    assert open(path, "rb").read() == ref


def test_tecplot_3d_bytes_match_reference(tmp_path):
    g = load_golden("ref3d_40x12x12")
    path = str(tmp_path / "out.plt")
    write_tecplot_fields(path, g["u"], g["v"], g["w"], g["p"], 1)
    ref = open(os.path.join(GOLDEN, "ref3d_40x12x12_output1.plt"), "rb").read()
    mine = open(path, "rb").read()
    assert len(mine) == len(ref) == 332 + 7 * 8 * 40 * 12 * 12
    assert mine == ref


def test_strouhal_of_a_pure_tone():
    n, period = 4000, 200.0
    t = np.arange(n)
    cl = 0.3 * np.sin(2 * np.pi * t / period) + 1e-3 * t / n
    st = cflbm.analysis.strouhal(cl, diam=20.0, u0=0.05)
    assert abs(st - 20.0 / period / 0.05) < 2e-3


def test_drag_over_whole_shedding_periods():
    """A window that ends mid-cycle moves the plain mean of a drag oscillating
    at twice the shedding frequency; the mean over whole periods (the period
    from the periodogram peak, within a fraction of a percent over 4.7 cycles)
    moves far less."""
    diam, u0, period = 20.0, 0.05, 2040.0
    n = int(4.7 * period)
    t = np.arange(n)
    q = 0.5 * u0 * u0 * diam
    cl = 0.5 * np.sin(2 * np.pi * t / period)
    cd = 1.82 + 0.05 * np.sin(4 * np.pi * t / period)
    force = np.stack([cd * q, cl * q, np.zeros(n)], axis=1)
    a, k = cflbm.analysis.shedding_window(cl, diam, u0)
    assert k == 4 and abs((n - a) - 4 * period) <= 0.005 * 4 * period
    st = cflbm.analysis.summary(force, u0, diam, diam, n)
    assert st["periods"] == 4
    assert abs(st["cd_mean"] - 1.82) > 1e-3  # the plain mean: 1.5e-3 off
    assert abs(st["cd_mean_periods"] - 1.82) < 2e-4
    # no oscillation: the whole-period mean falls back to the plain mean
    flat = np.stack([np.full(n, 1.5 * q), np.zeros(n), np.zeros(n)], axis=1)
    st0 = cflbm.analysis.summary(flat, u0, diam, diam, n)
    assert st0["periods"] == 0 and st0["cd_mean_periods"] == st0["cd_mean"]


def test_test_dat_format(tmp_path):
    p = str(tmp_path / "test.dat")
    cflbm.analysis.write_test_dat(p, np.array([[1.25, -0.5]]), append=False)
    assert open(p).read() == "1.25000000000000000 -0.50000000000000000\n"
