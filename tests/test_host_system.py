"""The drop-in System class (host/System.cpp) reads input.in as the reference's
System does: the derived values match the reference's own (golden
tests/golden/system_input.json, made by the reference compiled from its
sources), and the extension keys after the separator set the solver options.
Compiled here with the host C++ compiler; no GPU."""
from __future__ import annotations

import json
import os
import subprocess

import pytest

from conftest import GOLDEN, PKG, ROOT

HARNESS = r'''
#include <cstdio>
#include "System.hpp"
int main(int argc, char **argv) {
  System s(argv[1]);
  std::printf("%d %d %d %d %d %d %.17g %.17g %.17g %.17g %.17g %.17g %d\n", s.ok ? 1 : 0, s.sx,
              s.sy, s.sz, s.Time, s.inter, s.miu, s.u0, s.R, s.rho0, s.Ma, s.tau, s.Re);
  std::printf("%d %d %d %d %d %.17g %.17g %.17g %.17g %d %d %.17g %llu %d\n", s.lattice,
              s.profile, s.storage, s.compute, s.geom, s.cx, s.cy, s.cz, s.diam, s.wall_y,
              s.wall_z, s.perturb, (unsigned long long)s.seed, s.rounding);
  std::printf("%s\n", s.error.c_str());
  return 0;
}
'''


@pytest.fixture(scope="module")
def system_exe(tmp_path_factory):
    d = tmp_path_factory.mktemp("system")
    src = d / "h.cpp"
    src.write_text(HARNESS)
    exe = d / "h"
    host = os.path.join(PKG, "host")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", host, "-I", os.path.join(ROOT, "include"),
                    str(src), os.path.join(host, "System.cpp"), "-o", str(exe)], check=True)
    return str(exe)


def read(exe, path):
    out = subprocess.run([exe, str(path)], capture_output=True, text=True,
                         check=True).stdout.split("\n")
    return out[0].split(), out[1].split()


def read_error(exe, path):
    return subprocess.run([exe, str(path)], capture_output=True, text=True,
                          check=True).stdout.split("\n")[2]


def test_derived_values_match_the_reference_system(system_exe, tmp_path):
    g = json.load(open(os.path.join(GOLDEN, "system_input.json")))
    p = tmp_path / "input.in"
    p.write_text(g["input.in"])
    a, _ = read(system_exe, p)
    ref = g["system"]
    assert a[0] == "1"
    assert [int(v) for v in a[1:6]] == [ref["sx"], ref["sy"], ref["sz"], ref["Time"],
                                         ref["inter"]]
    for v, k in zip(a[6:12], ("miu", "u0", "R", "rho0", "Ma", "tau")):
        assert float(v) == pytest.approx(ref[k], rel=1e-15, abs=0), k
    assert int(a[12]) == ref["Re"]


def test_extension_keys_set_solver_options(system_exe, tmp_path):
    p = tmp_path / "input.in"
    p.write_text("1.0  8.0  100\n0.05  100  10\n400  100  1\n=============\nrho R Re\n"
                 "cflbm.lattice 9\ncflbm.profile channel\ncflbm.storage fp32\n"
                 "cflbm.compute fp32\ncflbm.steps 2000\ncflbm.inter 500\ncflbm.geom cylinder\n"
                 "cflbm.center 80 50 0\ncflbm.diam 20\ncflbm.wall_y noslip\n"
                 "cflbm.wall_z periodic\ncflbm.perturb 0.001\ncflbm.seed 99\n"
                 "cflbm.rounding nearest\n")
    a, b = read(system_exe, p)
    assert (int(a[4]), int(a[5])) == (2000, 500)
    assert b[:5] == ["9", "0", "1", "1", "1"]
    assert [float(v) for v in b[5:9]] == [80.0, 50.0, 0.0, 20.0]
    assert b[9:11] == ["1", "2"]
    assert float(b[11]) == 0.001 and b[12] == "99"
    assert b[13] == "0"  # CFLBM_ROUND_NEAREST (stochastic when the key is absent)


def test_missing_input_is_reported(system_exe, tmp_path):
    a, _ = read(system_exe, tmp_path / "does_not_exist.in")
    assert a[0] == "0"


def test_extension_key_selects_double_float_collision(system_exe, tmp_path):
    p = tmp_path / "input.in"
    p.write_text("1.0  8.0  100\n0.05  100  10\n64  32  32\n=============\nrho R Re\n"
                 "cflbm.compute df64\n")
    _, b = read(system_exe, p)
    assert b[1:4] == ["2", "0", "2"]  # profile REF3D, FP64 storage, double-float collision


@pytest.mark.parametrize("key,value", [("profile", "Channel"), ("storage", "fp16"),
                                       ("compute", "DF64"), ("geom", "disk"),
                                       ("wall_y", "slip"), ("wall_z", "wall"),
                                       ("rounding", "stochastic-ish")])
def test_unknown_extension_values_are_rejected(system_exe, tmp_path, key, value):
    p = tmp_path / "input.in"
    p.write_text("1.0  8.0  100\n0.05  100  10\n64  32  32\n=============\nrho R Re\n"
                 f"cflbm.{key} {value}\n")
    a, _ = read(system_exe, p)
    assert a[0] == "0"
    msg = read_error(system_exe, p)
    assert f"cflbm.{key}" in msg and value in msg


def test_unknown_extension_key_is_rejected(system_exe, tmp_path):
    p = tmp_path / "input.in"
    p.write_text("1.0  8.0  100\n0.05  100  10\n64  32  32\n=============\nrho R Re\n"
                 "cflbm.storag fp32\n")
    a, _ = read(system_exe, p)
    assert a[0] == "0"
    assert "cflbm.storag" in read_error(system_exe, p)
