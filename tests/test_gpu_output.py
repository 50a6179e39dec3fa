"""The reference's post-stream state and its ASCII Output files.

The reference's f holds, after Streaming() and Update(), the post-stream
(pre-collision) populations; its Output(n) writes population 1 of them in 3-D
("3D MPI+KOKKOS+MPIIO/lbm.cpp:741-771") and x, y, u, v, p in 2-D ("MPI
Kokkos/lbm.cpp:738-765").  The handle keeps the post-collision state, and
cflbm_get_f_stream forms the last step's pull.  Checked against the
reference's own outputs (golden fixtures from the compiled reference) and, for
the channel profile, against the oracle's post-stream state; and the drop-in
LBM class's Output files against the reference's files of the same run."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, PKG, ROOT, load_golden, rel_err
from oracle import oracle as O

from cflbm import Solver

pytestmark = pytest.mark.gpu


def test_ref2d_post_stream_state_matches_reference(cuda):
    g = load_golden("ref2d_96x40")
    m = g["meta"]
    with Solver(lattice=9, nx=m["nx"], ny=m["ny"], profile="ref2d", tau0=m["tau0"], u0=m["u0"],
                ref_ran=g["ran"]) as s:
        s.step(m["steps"])
        fs = s.get_f_stream()[:, 0]
    assert rel_err(fs, g["fstream"]) < 1e-11


def test_ref3d_post_stream_state_matches_reference(cuda):
    g = load_golden("ref3d_40x12x12")
    m = g["meta"]
    with Solver(lattice=27, nx=m["nx"], ny=m["ny"], nz=m["nz"], profile="ref3d",
                tau0=m["tau0"], u0=m["u0"], ref_ran=g["ran"]) as s:
        f0 = s.get_f()
        assert np.array_equal(s.get_f_stream(), f0)  # before any step: the initial feq
        s.step(m["steps"])
        fs = s.get_f_stream()
    assert rel_err(fs, g["fstream"]) < 1e-11


@pytest.mark.parametrize("lattice,wall_y,wall_z", [(9, "freeslip", "periodic"),
                                                   (9, "noslip", "periodic"),
                                                   (27, "freeslip", "periodic"),
                                                   (27, "noslip", "freeslip")])
def test_channel_post_stream_state_matches_oracle(cuda, lattice, wall_y, wall_z):
    nz = 12 if lattice == 27 else 1
    kw = dict(lattice=lattice, nx=72, ny=24, nz=nz, tau0=0.03, u0=0.05, wall_y=wall_y,
              wall_z=wall_z, geom="cylinder", cx=20, cy=12, diam=8, perturb_amp=1e-3, seed=7)
    steps = 15
    with Solver(**kw) as s:
        s.step(steps)
        fs = s.get_f_stream()
    W = {"freeslip": O.WALL_FREESLIP, "noslip": O.WALL_NOSLIP, "periodic": O.WALL_PERIODIC}
    cfg = O.channel_cfg(lattice, 72, 24, nz, tau0=0.03, u_in=0.05, wall_y=W[wall_y],
                        wall_z=W[wall_z], geom=O.GEOM_CYLINDER, cx=20, cy=12, diam=8, amp=1e-3,
                        seed=7)
    o = O.channel(cfg, steps, want_f=False, want_fstream=True)
    assert rel_err(fs, o["fstream"].reshape(fs.shape)) < 1e-10


HARNESS = r'''
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "lbm.hpp"
// dim nx ny nz tau0 u0 steps ranfile: the reference's loop with its Output(0)
// after Initialize and Output(1) after the run, on the drop-in class.
int main(int argc, char **argv) {
  const int dim = std::atoi(argv[1]), nx = std::atoi(argv[2]), ny = std::atoi(argv[3]),
            nz = std::atoi(argv[4]), steps = std::atoi(argv[7]);
  double tau = std::atof(argv[5]), u0 = std::atof(argv[6]), rho0 = 1.0;
  const int G = dim <= 2 ? 2 : 3;
  std::vector<int32_t> ran((size_t)(nx + 2 * G) * (ny + 2 * G) * (dim <= 2 ? 1 : nz + 2 * G));
  std::FILE *fp = std::fopen(argv[8], "rb");
  if (!fp || std::fread(ran.data(), 4, ran.size(), fp) != ran.size()) return 3;
  std::fclose(fp);
  // dim 1: the serial 2-D variant, LBM(sx, sy) with sx = nx - 1, sy = ny - 1
  LBM *l = dim == 1 ? new LBM(nx - 1, ny - 1, tau, rho0, u0)
           : dim == 2 ? new LBM(MPI_COMM_WORLD, nx, ny, tau, rho0, u0)
                      : new LBM(MPI_COMM_WORLD, nx, ny, nz, tau, rho0, u0);
  l->config.ref_ran = ran.data();
  l->Initialize();
  l->Output(0);
  for (int it = 1; it <= steps; ++it) {
    l->Collision();
    l->Streaming();
    l->Update();
  }
  l->Output(1);
  // the f, usr and rho views at an interior node next to the body's centre
  std::printf("%.17g %d %.17g\n", dim <= 2 ? l->f(1, G + 1, G + 1) : l->f(1, G + 1, G + 1, G + 1),
              dim == 1   ? l->usr((int)(0.25 * (nx - 1) + 0.5), (ny + 3) / 2)  // disk centre
              : dim == 2 ? l->usr(G + nx / 2, G + ny / 2)                     // disk centre
                         : l->usr(G + 1, G + 1, G + 1),
              dim <= 2 ? l->rho(G, G) : l->rho(G, G, G));
  delete l;
  return 0;
}
'''


@pytest.fixture(scope="module")
def output_exe(tmp_path_factory):
    d = tmp_path_factory.mktemp("output")
    src = d / "h.cpp"
    src.write_text(HARNESS)
    exe = d / "h"
    host = os.path.join(PKG, "host")
    lib = os.path.join(PKG, "cflbm")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", host, "-I", os.path.join(ROOT, "include"),
                    str(src), os.path.join(host, "libcflbm_host.a"), "-L", lib, "-lcflbm",
                    f"-Wl,-rpath,{lib}", "-o", str(exe)], check=True)
    return str(exe)


def _same_dat(mine: str, ref: str):
    """Byte-identical, except that a last printed digit may differ where the two
    FP64 values differ in their last bits (8 fixed decimals)."""
    a = open(mine).read().splitlines()
    b = open(ref).read().splitlines()
    assert len(a) == len(b)
    assert a[:2] == b[:2]
    diff = [(x, y) for x, y in zip(a[2:], b[2:]) if x != y]
    for x, y in diff:
        fx, fy = [float(t) for t in x.split()], [float(t) for t in y.split()]
        assert len(fx) == len(fy) and np.allclose(fx, fy, rtol=0, atol=1.01e-8), (x, y)
    assert len(diff) <= max(3, len(a) // 100), len(diff)


@pytest.mark.parametrize("name,dim", [("ref2d_96x40", 2), ("ref3d_40x12x12", 3),
                                      ("ref2ds_96x36", 1)])
def test_dropin_output_files_match_reference(cuda, output_exe, tmp_path, name, dim):
    g = load_golden(name)
    m = g["meta"]
    ranfile = tmp_path / "ran.i32"
    g["ran"].astype(np.int32).tofile(ranfile)
    r = subprocess.run([output_exe, str(dim), str(m["nx"]), str(m["ny"]), str(m.get("nz", 1)),
                        repr(m["tau0"]), repr(m["u0"]), str(m["steps"]), str(ranfile)],
                       cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    for k in (0, 1):
        if dim == 1:  # the serial variant's files are output<n>.dat
            _same_dat(str(tmp_path / f"output{k}.dat"), os.path.join(GOLDEN, f"{name}_output{k}.dat"))
        else:
            _same_dat(str(tmp_path / f"output{k}0.dat"),
                      os.path.join(GOLDEN, f"{name}_output{k}0.dat"))
    f1, usr, rho = r.stdout.split()[-3:]
    if dim <= 2:
        assert float(f1) == pytest.approx(g["fstream"][1, 1, 1], rel=1e-11, abs=1e-15)
        assert usr == "0"  # at the disk's centre
    else:
        assert float(f1) == pytest.approx(g["fstream"][1, 1, 1, 1], rel=1e-11, abs=1e-15)
        assert usr == "1"
    assert float(rho) == 1.0
