"""Accuracy/throughput studies of the storage and arithmetic forms.

precision_study: one problem run with FP64 arithmetic on FP64 storage (the
reference arithmetic, used as the FP64 oracle at sizes the CPU oracle cannot
reach) and with FP32 arithmetic on FP64, FP32 and FP16-deviation storage.  For
each form it reports the sweep's MLUPS and HBM fraction, the final u field's
error against the FP64 run, the mean drag coefficient, its error, the lift rms,
the Strouhal number and the FP64 mass drift.

    python -m cflbm.studies precision --nx 768 --ny 384 --nz 384 --steps 20000
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import analysis
from .solver import Solver

FORMS = [  # name, storage, compute
    ("fp64_arith", "fp64", "fp64"),
    ("fp64_store", "fp64", "fp32"),
    ("fp32_store", "fp32", "fp32"),
    ("fp16dev_store", "fp16dev", "fp32"),
]


def sphere_case(nx=768, ny=384, nz=384, diam=64.0, u0=0.03, re=300.0):
    """The precision-form problem: a sphere in a free-slip box."""
    return dict(lattice=27, nx=nx, ny=ny, nz=nz, tau0=3.0 * u0 * diam / re, u0=u0,
                wall_y="freeslip", wall_z="freeslip", geom="sphere", cx=nx / 4.0,
                cy=ny / 2.0, cz=nz / 2.0, diam=diam, perturb_amp=1e-3, seed=1234)


def run_form(case, storage, compute, steps, window, peak_gbs, chunk=1000, timing_steps=20):
    out = {}
    with Solver(storage=storage, compute=compute, force_history=steps + 8, **case) as s:
        info = s.info()
        m0, _ = s.mass()
        t0 = time.perf_counter()
        done = 0
        while done < steps:
            n = min(chunk, steps - done)
            s.step(n)
            done += n
        s.synchronize()
        wall = time.perf_counter() - t0
        m1, _ = s.mass()
        u = s.macros()[0]
        hist = s.force_history(steps)
        s.set_timing(True)
        s.step(timing_steps)
        sw_ms, _, n_sw, _ = s.timing()
        cells = case["nx"] * case["ny"] * case["nz"]
        area = np.pi * case["diam"] ** 2 / 4.0 if case["geom"] == "sphere" else (
            case["diam"] * (case["nz"] if case["lattice"] == 27 else 1))
        st = analysis.summary(hist, case["u0"], area, case["diam"], window)
        sweep_s = sw_ms * 1e-3 / max(n_sw, 1)
        out.update(
            mlups_wall=cells * steps / wall / 1e6,
            mlups_sweep=cells / sweep_s / 1e6,
            hbm_frac=info.bytes_per_cell_step * cells / sweep_s / 1e9 / peak_gbs,
            bytes_per_cell=info.bytes_per_cell_step,
            mass_drift=(m1 - m0) / m0, **st)
    return out, u


def precision_study(case, steps, window, peak_gbs, forms=FORMS, out_path=None):
    results = {"case": case, "steps": steps, "window": window, "forms": {}}
    u_ref = None
    cd_ref = None
    for name, storage, compute in forms:
        r, u = run_form(case, storage, compute, steps, window, peak_gbs)
        if u_ref is None:
            u_ref, cd_ref = u, r["cd_mean"]
        r["u_err_linf"] = float(np.max(np.abs(u - u_ref)) / np.max(np.abs(u_ref)))
        r["u_err_l2"] = float(np.linalg.norm(u - u_ref) / np.linalg.norm(u_ref))
        r["cd_err_abs"] = float(abs(r["cd_mean"] - cd_ref))
        r["cd_err_rel"] = float(abs(r["cd_mean"] - cd_ref) / abs(cd_ref))
        results["forms"][name] = r
        del u
        if out_path:
            with open(out_path, "w") as fh:
                json.dump(results, fh, indent=1)
        print(name, json.dumps(r), flush=True)
    return results


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("study", choices=["precision"])
    ap.add_argument("--nx", type=int, default=768)
    ap.add_argument("--ny", type=int, default=384)
    ap.add_argument("--nz", type=int, default=384)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--window", type=int, default=5000)
    ap.add_argument("--peak", type=float, default=6656.0)
    ap.add_argument("--out", default=None)
    ap.add_argument("--forms", default=",".join(f[0] for f in FORMS))
    args = ap.parse_args()
    keep = set(args.forms.split(","))
    forms = [f for f in FORMS if f[0] in keep]
    case = sphere_case(args.nx, args.ny, args.nz, diam=64.0 * args.nx / 768.0)
    precision_study(case, args.steps, args.window, args.peak, forms, args.out)


if __name__ == "__main__":
    main()
