"""Build the C++ drop-in driver (System/LBM classes + the reference's main loop).

Produces host/cflbm_main, linked against cflbm/libcflbm.so (rpath $ORIGIN/../cflbm),
and host/libcflbm_host.a with the System/LBM classes for callers that bring their
own main().
"""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIBDIR = os.path.join(ROOT, "cflbm")
BUILD = os.path.join(ROOT, "_build")
FLAGS = ["-std=c++17", "-O2", "-ffp-contract=off", "-Wall"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build() -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, f) for f in ("System.cpp", "lbm.cpp")]
    objs = []
    for s in srcs:
        o = os.path.join(BUILD, "host_" + os.path.basename(s) + ".o")
        _run(["g++", *FLAGS, "-fPIC", "-c", s, "-o", o])
        objs.append(o)
    lib = os.path.join(HERE, "libcflbm_host.a")
    if os.path.exists(lib):
        os.remove(lib)
    _run(["ar", "rcs", lib, *objs])
    exe = os.path.join(HERE, "cflbm_main")
    _run(["g++", *FLAGS, os.path.join(HERE, "main.cpp"), lib, "-L", LIBDIR, "-lcflbm",
          "-Wl,-rpath,$ORIGIN/../cflbm", "-o", exe])
    return exe


if __name__ == "__main__":
    print(build())
