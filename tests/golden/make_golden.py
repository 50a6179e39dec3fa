"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs the reference's own sources (compiled unmodified against the Kokkos/MPI
shim by oracle/build.py into oracle/_ref/) on small grids and stores what they
produce: the per-node random draw, the post-collision populations and the
macroscopic fields of the interior, the post-stream populations (the
reference's f after Update), the per-step "Cd Cl" lines of test.dat, the
Tecplot files written by MPIoutput, the ASCII files written by Output, and the
parameters System derives from an input.in.  Needs the reference checkout; the fixtures are committed so the GPU
box (which has no reference) can check against them.

    python tests/golden/make_golden.py [ref2d_96x40 ref3d_40x12x12 ref2ds_96x36 system_input]
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build as obuild  # noqa: E402
from oracle import oracle as O  # noqa: E402

CASES_2D = [dict(name="ref2d_96x40", nx=96, ny=40, tau0=0.03, u0=0.05, steps=200)]
CASES_3D = [dict(name="ref3d_40x12x12", nx=40, ny=12, nz=12, tau0=0.0192, u0=0.04, steps=40)]
# the serial "Kokkos/" variant: LBM(sx, sy) has (sx + 1) x (sy + 1) interior nodes
CASES_2DS = [dict(name="ref2ds_96x36", nx=96, ny=36, sx=95, sy=35, tau0=0.03, u0=0.05,
                  steps=150)]
INPUT_IN = "1.0  8.0  100\n0.1  100  10\n512  128  128\n=============\nrho R Re\nu0 Time inter\nnx ny nz\n"


def main(only: list[str]) -> None:
    if not obuild.reference_available():
        raise SystemExit("the reference checkout is needed to regenerate the fixtures")
    obuild.build_ref()
    want = (lambda name: not only or name in only)  # noqa: E731
    for c in CASES_2DS:
        if not want(c["name"]):
            continue
        r = O.run_ref2ds_binary(c["sx"], c["sy"], c["tau0"], c["u0"], c["steps"])
        G = 2
        sl = (slice(G, G + c["nx"]), slice(G, G + c["ny"]))
        np.savez_compressed(
            os.path.join(HERE, c["name"] + ".npz"),
            meta=json.dumps(c), ran=r["ran"],
            fpost=r["fpost"][(slice(None),) + sl].transpose(0, 2, 1),
            u=r["u"][sl].T, v=r["v"][sl].T, p=r["p"][sl].T,
            fstream=r["f"][(slice(None),) + sl].transpose(0, 2, 1))
        for k in (0, 1):
            src = os.path.join(r["dir"], f"output{k}.dat")
            with open(src, "rb") as fh, open(os.path.join(HERE, f"{c['name']}_output{k}.dat"), "wb") as out:
                out.write(fh.read())
    for c in CASES_2D:
        if not want(c["name"]):
            continue
        r = O.run_ref2d_binary(c["nx"], c["ny"], c["tau0"], c["u0"], c["steps"])
        G = 2
        sl = (slice(G, G + c["nx"]), slice(G, G + c["ny"]))
        cdcl = np.loadtxt(os.path.join(r["dir"], "test.dat")).reshape(-1, 2)
        np.savez_compressed(
            os.path.join(HERE, c["name"] + ".npz"),
            meta=json.dumps(c), ran=r["ran"],
            # interior, transposed to x fastest: [.., y, x]
            fpost=r["fpost"][(slice(None),) + sl].transpose(0, 2, 1),
            u=r["u"][sl].T, v=r["v"][sl].T, p=r["p"][sl].T, cdcl=cdcl,
            # the post-stream state after the run (the reference's f after Update)
            fstream=r["f"][(slice(None),) + sl].transpose(0, 2, 1))
        for k in (0, 1):
            src = os.path.join(r["dir"], f"output{k}0.dat")
            with open(src, "rb") as fh, open(os.path.join(HERE, f"{c['name']}_output{k}0.dat"), "wb") as out:
                out.write(fh.read())
        for k in (0, 1):
            src = os.path.join(r["dir"], f"output{k}.plt")
            with open(src, "rb") as fh, open(os.path.join(HERE, f"{c['name']}_output{k}.plt"), "wb") as out:
                out.write(fh.read())
    for c in CASES_3D:
        if not want(c["name"]):
            continue
        r = O.run_ref3d_binary(c["nx"], c["ny"], c["nz"], c["tau0"], c["u0"], c["steps"])
        G = 3
        sl = (slice(G, G + c["nx"]), slice(G, G + c["ny"]), slice(G, G + c["nz"]))
        np.savez_compressed(
            os.path.join(HERE, c["name"] + ".npz"),
            meta=json.dumps(c), ran=r["ran"],
            fpost=r["fpost"][(slice(None),) + sl].transpose(0, 3, 2, 1),
            u=r["u"][sl].transpose(2, 1, 0), v=r["v"][sl].transpose(2, 1, 0),
            w=r["w"][sl].transpose(2, 1, 0), p=r["p"][sl].transpose(2, 1, 0),
            fstream=r["f"][(slice(None),) + sl].transpose(0, 3, 2, 1))
        for k in (0, 1):
            src = os.path.join(r["dir"], f"output{k}0.dat")
            with open(src, "rb") as fh, open(os.path.join(HERE, f"{c['name']}_output{k}0.dat"), "wb") as out:
                out.write(fh.read())
        src = os.path.join(r["dir"], "output1.plt")
        with open(src, "rb") as fh, open(os.path.join(HERE, f"{c['name']}_output1.plt"), "wb") as out:
            out.write(fh.read())
    if not want("system_input"):
        print("fixtures written to", HERE)
        return
    # System's parameter derivation from input.in.
    d = tempfile.mkdtemp(prefix="sys_")
    with open(os.path.join(d, "input.in"), "w") as fh:
        fh.write(INPUT_IN)
    out = subprocess.run([O.ref_binary("ref3d"), "system", d], check=True, capture_output=True,
                         text=True).stdout
    with open(os.path.join(HERE, "system_input.json"), "w") as fh:
        json.dump({"input.in": INPUT_IN, "system": json.loads(out)}, fh, indent=1)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main(sys.argv[1:])  # fixture names to regenerate (default: all)
