"""The reference's 3-D driver loop on the drop-in classes (host/cflbm_main:
System reads input.in, LBM steps, MPIoutput every `inter` steps) writes the same
Tecplot files, byte for byte, as the library does for the same run."""
from __future__ import annotations

import os
import subprocess

import pytest

from conftest import PKG

from cflbm import Solver

pytestmark = pytest.mark.gpu


def test_host_driver_writes_what_the_library_writes(cuda, tmp_path):
    exe = os.path.join(PKG, "host", "cflbm_main")
    assert os.path.exists(exe), "host/cflbm_main is built by __graft_entry__.build()"
    # rho R Re / u0 Time inter / nx ny nz as the reference reads them; tau =
    # u0 R / Re / cs2 = 0.024; the run length comes from the extension keys.
    (tmp_path / "input.in").write_text(
        "1.0  8.0  100\n0.1  100  10\n40  12  12\n=============\nrho R Re\nu0 Time inter\n"
        "nx ny nz\ncflbm.steps 40\ncflbm.inter 20\n")
    r = subprocess.run([exe], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert r.stdout.count("time=") == 2
    with Solver(lattice=27, nx=40, ny=12, nz=12, profile="ref3d", tau0=0.024, u0=0.1) as s:
        for n in range(3):
            if n:
                s.step(20)
            mine = tmp_path / f"lib{n}.plt"
            s.write_tecplot(str(mine), n)
            assert (tmp_path / f"output{n}.plt").read_bytes() == mine.read_bytes(), n
