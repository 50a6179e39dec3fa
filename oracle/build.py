"""Build recipe for the CPU oracle: TEST INFRASTRUCTURE ONLY.

* ``build_oracle()`` compiles oracle/lbm_oracle.cpp (the FP64 C++/OpenMP
  restatement of the reference) into oracle/liboracle.so.
* ``build_ref()`` compiles the reference's own, unmodified sources from
  ``/root/reference`` against the Kokkos/MPI subset shim in oracle/shim/ into
  oracle/_ref/ref2d, oracle/_ref/ref3d and oracle/_ref/ref2ds (the serial
  "Kokkos/" variant) (drivers: oracle/ref_driver_*.cpp).
  It needs the reference checkout and is skipped where that is absent.

Both use the same flags (-O3, no fast-math, -ffp-contract=off), so the
restatement and the compiled reference agree bit for bit.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE = os.environ.get("CFLBM_REFERENCE_DIR", "/root/reference")
CXXFLAGS = ["-std=c++17", "-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math"]


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stale(out: str, srcs: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs if os.path.exists(s))


def oracle_lib_path() -> str:
    return os.path.join(HERE, "liboracle.so")


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "lbm_oracle.cpp")
    out = oracle_lib_path()
    if force or _stale(out, [src, __file__]):
        _run(["g++", *CXXFLAGS, "-shared", "-fPIC", src, "-o", out])
    return out


def reference_available() -> bool:
    return all(os.path.isdir(os.path.join(REFERENCE, d))
               for d in ("MPI Kokkos", "3D MPI+KOKKOS+MPIIO", "Kokkos"))


def build_ref(force: bool = False) -> list[str]:
    """Compile the reference sources (unmodified) with the shim into oracle/_ref/."""
    if not reference_available():
        return []
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    shim = os.path.join(HERE, "shim")
    shim_hdrs = [os.path.join(shim, h) for h in os.listdir(shim)]
    d2 = os.path.join(REFERENCE, "MPI Kokkos")
    d3 = os.path.join(REFERENCE, "3D MPI+KOKKOS+MPIIO")
    jobs = []
    src2 = [os.path.join(HERE, "ref_driver_2d.cpp"), os.path.join(d2, "lbm.cpp")]
    out2 = os.path.join(outdir, "ref2d")
    if force or _stale(out2, src2 + shim_hdrs):
        jobs.append(["g++", *CXXFLAGS, "-w", "-I", shim, "-I", d2, *src2, "-o", out2])
    src3 = [os.path.join(HERE, "ref_driver_3d.cpp"), os.path.join(d3, "lbm.cpp"),
            os.path.join(d3, "System.cpp")]
    out3 = os.path.join(outdir, "ref3d")
    if force or _stale(out3, src3 + shim_hdrs):
        jobs.append(["g++", *CXXFLAGS, "-w", "-I", shim, "-I", d3, *src3, "-o", out3])
    d2s = os.path.join(REFERENCE, "Kokkos")
    src2s = [os.path.join(HERE, "ref_driver_2ds.cpp"), os.path.join(d2s, "lbm.cpp")]
    out2s = os.path.join(outdir, "ref2ds")
    if force or _stale(out2s, src2s + shim_hdrs):
        jobs.append(["g++", *CXXFLAGS, "-w", "-I", shim, "-I", d2s, *src2s, "-o", out2s])
    with ThreadPoolExecutor(max_workers=3) as ex:
        list(ex.map(_run, jobs))
    return [out2, out3, out2s]


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
