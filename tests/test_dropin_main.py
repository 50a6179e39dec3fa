"""The reference's own 3-D driver ("3D MPI+KOKKOS+MPIIO/main.cpp"), compiled
unmodified against the drop-in classes (host/lbm.hpp, host/System.hpp) and the
single-rank MPI and Kokkos stand-ins (host/mpi.h, host/Kokkos_Core.hpp), links
against libcflbm.so and reads input.in through the drop-in System.  The file is
fed to the compiler on standard input so its quoted includes resolve to the
drop-in headers rather than to the reference's own next to it; nothing is
copied.  Needs the reference checkout (absent on GPU machines); no GPU."""
from __future__ import annotations

import os
import subprocess

import pytest

from conftest import PKG, ROOT
from oracle import build as obuild

MAIN = os.path.join(obuild.REFERENCE, "3D MPI+KOKKOS+MPIIO", "main.cpp")
pytestmark = pytest.mark.skipif(not os.path.exists(MAIN), reason="reference checkout absent")


@pytest.fixture(scope="module")
def ref_main(tmp_path_factory):
    host = os.path.join(PKG, "host")
    lib = os.path.join(PKG, "cflbm")
    assert os.path.exists(os.path.join(host, "libcflbm_host.a")), "built by build()"
    d = tmp_path_factory.mktemp("refmain")
    exe = d / "ref_main"
    with open(MAIN, "rb") as src:
        r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", host, "-I",
                            os.path.join(ROOT, "include"), "-x", "c++", "-", "-x", "none",
                            os.path.join(host, "libcflbm_host.a"), "-L", lib, "-lcflbm",
                            f"-Wl,-rpath,{lib}", "-o", str(exe)],
                           stdin=src, capture_output=True, text=True, cwd=d)
    assert r.returncode == 0, r.stderr
    return exe


def test_reference_main_compiles_and_links(ref_main):
    assert os.access(ref_main, os.X_OK)


def test_reference_main_reads_input_through_the_dropin(ref_main, tmp_path):
    # A misspelt extension value stops the drop-in LBM before any device call,
    # with a message that names the key (System prints its banner first).
    (tmp_path / "input.in").write_text(
        "1.0  8.0  100\n0.1  100  10\n40  12  12\n=============\ncflbm.storage fp16\n")
    r = subprocess.run([str(ref_main)], cwd=tmp_path, capture_output=True, text=True,
                       timeout=60)
    assert r.returncode != 0
    assert "3D Cylinder Flow" in r.stdout and "nx    =40" in r.stdout
    assert "cflbm.storage" in r.stderr and "fp16" in r.stderr
