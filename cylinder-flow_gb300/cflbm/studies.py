"""Accuracy/throughput studies of the storage and arithmetic forms.

precision_study: one problem run with FP64 arithmetic on FP64 storage (the
reference arithmetic, used as the FP64 oracle at sizes the CPU oracle cannot
reach), with double-float (DF64) arithmetic on FP64 storage, and with FP32
arithmetic on FP64, FP32 and FP16-deviation storage.  For each form it reports
the sweep's MLUPS and HBM fraction, the final u field's error against the FP64
run, the mean drag coefficient (plain window mean and the mean over whole
shedding periods), their errors, the lift rms, the Strouhal number and the
FP64 mass drift.

    python -m cflbm.studies precision --nx 768 --ny 384 --nz 384 --steps 20000
    python -m cflbm.studies precision --case channel2d --steps 40000 --window 10000

The second line is the D2Q9 400x100 cylinder channel (Re 100) run to its
periodic state: its shedding grows until about step 28,000, so drag averaged
over steps 10,000-20,000 also measures when the shedding set in (which round-off
noise moves), while steps 30,000-40,000 measure the periodic state itself.

adjoint_study: the differentiation problem (D2Q9 1024x256 channel, cylinder
D=32 at (200, 128), porosity on a 128x128 box, mean drag over steps 5000-7000
of 7000, checkpoints every 100).  Runs the FP32 and FP64 adjoints, compares
them, and checks the FP64 gradient against central differences (h = 1e-4) of
the FP64 solver for u_in, tau and 16 seeded porosity directions; along each
direction also at 2h, and the Richardson extrapolation of the two.

    python -m cflbm.studies adjoint --out adjoint.json

batch_study: the batched form (64 D2Q9 cylinder channels, widths 256-1024 and
heights 64-256 in multiples of 32, D in [8, 32], Re in [40, 200], u_in = 0.05,
FP32 storage, 20000 steps in one launch per step over all channels, replayed
from a 100-step CUDA graph, autotuned launch shape) against the same channels run one
at a time with FP32 storage and arithmetic (the gain from batching alone) and
with FP64 storage and arithmetic (the plain drop-in); per-instance Cd error
against that FP64 run.

    python -m cflbm.studies batch --out batch.json
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import analysis
from .solver import Solver

def measured_peak_gbs() -> float:
    """HBM copy peak of this pool (MEASURED_PEAKS.json at the repository root),
    else the 6800 GB/s fallback of an earlier GB300 measurement."""
    import os
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(
        os.path.abspath(__file__)))), "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            return float(json.load(fh)["hbm_gbs"])
    return 6800.0


FORMS = [  # name, storage, compute, FP16 rounding
    ("fp64_arith", "fp64", "fp64", "nearest"),
    ("df64_arith", "fp64", "df64", "nearest"),
    ("fp64_store", "fp64", "fp32", "nearest"),
    ("fp32_store", "fp32", "fp32", "nearest"),
    ("fp16dev_store", "fp16dev", "fp32", "stochastic"),
    ("fp16dev_rn_store", "fp16dev", "fp32", "nearest"),
]


def sphere_case(nx=768, ny=384, nz=384, diam=64.0, u0=0.03, re=300.0, seed=1234):
    """The precision-form problem: a sphere in a free-slip box."""
    return dict(lattice=27, nx=nx, ny=ny, nz=nz, tau0=3.0 * u0 * diam / re, u0=u0,
                wall_y="freeslip", wall_z="freeslip", geom="sphere", cx=nx / 4.0,
                cy=ny / 2.0, cz=nz / 2.0, diam=diam, perturb_amp=1e-3, seed=seed)


def channel2d_case(nx=400, ny=100, diam=20.0, u0=0.05, re=100.0, seed=1234):
    """The small benchmark problem: a cylinder at (80, 50) in a free-slip channel."""
    return dict(lattice=9, nx=nx, ny=ny, nz=1, tau0=3.0 * u0 * diam / re, u0=u0,
                wall_y="freeslip", geom="cylinder", cx=nx / 5.0, cy=ny / 2.0, diam=diam,
                perturb_amp=1e-3, seed=seed)


def run_form(case, storage, compute, steps, window, peak_gbs, chunk=1000, timing_steps=20,
             rounding="nearest"):
    out = {}
    with Solver(storage=storage, compute=compute, rounding=rounding, force_history=steps + 8,
                **case) as s:
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
    ref = None
    for name, storage, compute, rounding in forms:
        r, u = run_form(case, storage, compute, steps, window, peak_gbs, rounding=rounding)
        if u_ref is None:
            u_ref, ref = u, dict(r)
        r["u_err_linf"] = float(np.max(np.abs(u - u_ref)) / np.max(np.abs(u_ref)))
        r["u_err_l2"] = float(np.linalg.norm(u - u_ref) / np.linalg.norm(u_ref))
        for k in ("cd_mean", "cd_mean_periods", "cl_rms", "st"):
            r[k + "_err_abs"] = float(abs(r[k] - ref[k]))
            r[k + "_err_rel"] = float(abs(r[k] - ref[k]) / max(abs(ref[k]), 1e-300))
        results["forms"][name] = r
        del u
        if out_path:
            with open(out_path, "w") as fh:
                json.dump(results, fh, indent=1)
        print(name, json.dumps(r), flush=True)
    return results


def adjoint_case(nx=1024, ny=256, diam=32.0, cx=200.0, cy=128.0, u0=0.05, re=100.0):
    """The differentiation problem (free-slip walls; tau = 0.5 + 3 u D / Re)."""
    return dict(lattice=9, nx=nx, ny=ny, geom="cylinder", cx=cx, cy=cy, diam=diam,
                wall_y="freeslip", perturb_amp=1e-3, seed=1234), u0, 0.5 + 3.0 * u0 * diam / re


def adjoint_study(steps=7000, window=(5000, 7000), checkpoint_every=100, box=128,
                  directions=16, h=1e-4, seed=11, out_path=None, nx=1024, ny=256,
                  precisions=("fp32", "fp64"), fd=True):
    from .adjoint import run, smooth_porosity
    case, u_in, tau = adjoint_case(nx=nx, ny=ny)
    x0, y0 = int(case["cx"]) - box // 2, int(case["cy"]) - box // 2
    alpha = smooth_porosity(nx, ny, (x0, y0, x0 + box, y0 + box), seed=seed)
    alpha = alpha.astype(np.float32).astype(np.float64)  # the solver stores FP32
    res = {"case": case, "u_in": u_in, "tau": tau, "steps": steps, "window": window,
           "checkpoint_every": checkpoint_every, "h": h}

    def dump():
        if out_path:
            with open(out_path, "w") as fh:
                json.dump(res, fh, indent=1)

    grads = {}
    for prec in precisions:
        c = dict(case, storage=prec, compute=prec)
        r = run(c, alpha, u_in, tau, steps, checkpoint_every, window)
        # plain forward step time of the same problem (graph replay, no checkpoints)
        with Solver(**c, u0=u_in, tau0=tau - 0.5, alpha=alpha, force_history=64) as s:
            s.step(200)
            s.synchronize()
            t0 = time.perf_counter()
            s.step(2000)
            s.synchronize()
            fwd_step = (time.perf_counter() - t0) / 2000
        grads[prec] = r
        res[prec] = {"J": r["J"], "dJ_du_in": r["dJ_du_in"], "dJ_dtau": r["dJ_dtau"],
                     "dJ_dalpha_norm": float(np.linalg.norm(r["dJ_dalpha"])),
                     "seconds_forward": r["seconds_forward"],
                     "seconds_reverse": r["seconds_reverse"],
                     "forward_step_s": fwd_step,
                     "reverse_step_s": r["seconds_reverse"] / steps,
                     "reverse_over_forward_step": r["seconds_reverse"] / steps / fwd_step,
                     "device_bytes": r["device_bytes"]}
        print(prec, json.dumps(res[prec]), flush=True)
        dump()
    if not fd or len(grads) < 2:
        dump()
        return res
    g64, g32 = grads["fp64"], grads["fp32"]
    res["fp32_vs_fp64"] = {
        "J_rel": abs(g32["J"] - g64["J"]) / abs(g64["J"]),
        "dJ_du_in_rel": abs(g32["dJ_du_in"] - g64["dJ_du_in"]) / abs(g64["dJ_du_in"]),
        "dJ_dtau_rel": abs(g32["dJ_dtau"] - g64["dJ_dtau"]) / abs(g64["dJ_dtau"]),
        "dJ_dalpha_rel_l2": float(np.linalg.norm(g32["dJ_dalpha"] - g64["dJ_dalpha"]) /
                                  np.linalg.norm(g64["dJ_dalpha"]))}
    print("fp32_vs_fp64", json.dumps(res["fp32_vs_fp64"]), flush=True)

    c64 = dict(case, storage="fp64", compute="fp64")

    def J(a, u, t):
        with Solver(**c64, u0=u, tau0=t - 0.5, alpha=a, force_history=steps) as s:
            s.step(steps)
            f = s.force_history(steps)
        return float(np.mean(f[window[0] - 1:window[1], 0]))

    fd = {}
    fd["dJ_du_in"] = (J(alpha, u_in + h, tau) - J(alpha, u_in - h, tau)) / (2 * h)
    fd["dJ_dtau"] = (J(alpha, u_in, tau + h) - J(alpha, u_in, tau - h)) / (2 * h)
    fd["dJ_du_in_rel_err"] = abs(g64["dJ_du_in"] - fd["dJ_du_in"]) / abs(fd["dJ_du_in"])
    fd["dJ_dtau_rel_err"] = abs(g64["dJ_dtau"] - fd["dJ_dtau"]) / abs(fd["dJ_dtau"])
    rng = np.random.default_rng(seed + 1)
    mask = np.zeros_like(alpha)
    mask[y0:y0 + box, x0:x0 + box] = 1.0
    dirs = []
    for k in range(directions):
        d = rng.standard_normal(alpha.shape) * mask
        d /= np.max(np.abs(d))
        # central differences at h and 2h along d, each divided by its own
        # (FP32-rounded) step so they estimate the same derivative dJ/dalpha . d;
        # Richardson's (4 D(h) - D(2h)) / 3 removes their h^2 truncation term
        dd = []
        for hk in (h, 2 * h):
            ap = (alpha + hk * d).astype(np.float32).astype(np.float64)
            am = (alpha - hk * d).astype(np.float32).astype(np.float64)
            step = ap - am
            dd.append(((J(ap, u_in, tau) - J(am, u_in, tau)) / (2 * hk),
                       float(np.sum(g64["dJ_dalpha"] * step)) / (2 * hk),
                       float(np.sum(g32["dJ_dalpha"] * step)) / (2 * hk)))
        (f1, a64, a32), (f2, a64b, _) = dd
        # the Richardson combination of the adjoint projections (the FP32 rounding
        # of the two steps differs slightly) against that of the differences
        fr = (4 * f1 - f2) / 3
        ar = (4 * a64 - a64b) / 3
        dirs.append({"fd_h": f1, "fd_2h": f2, "fd_richardson": fr, "adjoint_fp64": a64,
                     "adjoint_fp32": a32,
                     "rel_err_fp64_h": abs(a64 - f1) / abs(f1),
                     "rel_err_fp64": abs(ar - fr) / abs(fr),
                     "rel_err_fp32": abs(a32 - f1) / abs(f1)})
    fd["directions"] = dirs
    fd["max_rel_err_fp64_h"] = max(d["rel_err_fp64_h"] for d in dirs)
    fd["max_rel_err_fp64"] = max(d["rel_err_fp64"] for d in dirs)
    fd["median_rel_err_fp64"] = float(np.median([d["rel_err_fp64"] for d in dirs]))
    fd["max_rel_err_fp32"] = max(d["rel_err_fp32"] for d in dirs)
    res["finite_differences"] = fd
    print("fd", json.dumps({k: v for k, v in fd.items() if k != "directions"}), flush=True)
    dump()
    return res


def batch_cases(n=64, seed=2025, u0=0.05):
    """The batched-form channels: seeded uniform draws of width, height, diameter
    and Reynolds number; body at (4D, H/2); free-slip walls."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        nx = int(rng.integers(256 // 32, 1024 // 32 + 1)) * 32
        ny = int(rng.integers(64 // 32, 256 // 32 + 1)) * 32
        d = float(rng.uniform(8.0, 32.0))
        re = float(rng.uniform(40.0, 200.0))
        out.append(dict(lattice=9, nx=nx, ny=ny, tau0=3.0 * u0 * d / re, u0=u0,
                        wall_y="freeslip", geom="cylinder", cx=4.0 * d, cy=ny / 2.0, diam=d,
                        perturb_amp=1e-3, seed=1000 + k, re=re))
    return out


def batch_study(n=64, steps=20000, graph_steps=100, window=10000, peak_gbs=None,
                out_path=None, sequential=True, shape=None):
    """`shape` = (tile height, blocks per SM) fixes the launch shape instead of
    autotuning it (blocks per SM 0: one interior work item per block)."""
    from .solver import Batch
    if peak_gbs is None:
        peak_gbs = measured_peak_gbs()
    cases = batch_cases(n)
    cfgs = [{k: v for k, v in c.items() if k != "re"} for c in cases]
    cells = sum(c["nx"] * c["ny"] for c in cfgs)
    res = {"instances": n, "steps": steps, "graph_steps": graph_steps, "cells": cells,
           "cases": cases}
    t0 = time.perf_counter()
    kw = dict(autotune=True) if shape is None else dict(
        autotune=False, tile_height=shape[0], blocks_per_sm=shape[1])
    with Batch([dict(c, storage="fp32", compute="fp32", force_history=steps + 8)
                for c in cfgs], graph_steps=graph_steps, **kw) as b:
        t_create = time.perf_counter() - t0
        b.step(graph_steps)  # first replay captures the graph
        b.synchronize()
        t1 = time.perf_counter()
        b.step(steps - graph_steps)
        b.synchronize()
        wall = time.perf_counter() - t1
        info = b.info()
        cd32 = []
        for k, c in enumerate(cfgs):
            hist = b.instance(k).force_history(steps)
            cd32.append(analysis.summary(hist, c["u0"], c["diam"], c["diam"], window)["cd_mean"])
    bpc = info.bytes_per_cell_step
    res["batch"] = {
        "create_s": t_create, "wall_s": wall, "timed_steps": steps - graph_steps,
        "mlups": cells * (steps - graph_steps) / wall / 1e6,
        "hbm_frac": bpc * cells * (steps - graph_steps) / wall / 1e9 / peak_gbs,
        "bytes_per_cell_step": bpc, "tile_height": info.tile_height,
        "grid_blocks": info.grid_blocks, "tuned_candidates": info.tuned_candidates,
        "tuned_step_ms": info.tuned_step_ms}
    print("batch", json.dumps(res["batch"]), flush=True)
    if out_path:
        with open(out_path, "w") as fh:
            json.dump(res, fh, indent=1)
    if not sequential:
        return res
    def sequential(storage, compute):
        """The same channels one at a time (each its own graph-replayed step
        loop), and each one's mean drag over the window."""
        wall, cds = 0.0, []
        for c in cfgs:
            with Solver(**c, storage=storage, compute=compute, force_history=steps + 8) as s:
                s.synchronize()
                t = time.perf_counter()
                s.step(steps)
                s.synchronize()
                wall += time.perf_counter() - t
                hist = s.force_history(steps)
                b = s.info().bytes_per_cell_step
            cds.append(analysis.summary(hist, c["u0"], c["diam"], c["diam"], window)["cd_mean"])
        return {"wall_s": wall, "mlups": cells * steps / wall / 1e6,
                "hbm_frac": b * cells * steps / wall / 1e9 / peak_gbs}, cds

    # the gain from batching alone: the same FP32 storage and arithmetic, one
    # channel at a time; then the plain FP64 drop-in, the Cd reference
    res["sequential_fp32"], cd32s = sequential("fp32", "fp32")
    res["speedup_vs_fp32_sequential"] = res["batch"]["mlups"] / res["sequential_fp32"]["mlups"]
    res["cd_fp32_batch_vs_sequential_max_abs"] = max(abs(a - b) for a, b in zip(cd32, cd32s))
    print("sequential_fp32", json.dumps(res["sequential_fp32"]), flush=True)
    res["sequential_fp64"], cd64 = sequential("fp64", "fp64")
    err = [abs(a - b) / abs(b) for a, b in zip(cd32, cd64)]
    res["speedup"] = res["batch"]["mlups"] / res["sequential_fp64"]["mlups"]
    res["cd"] = {"fp32_batch": cd32, "fp64_sequential": cd64, "rel_err": err,
                 "max_rel_err": max(err), "median_rel_err": float(np.median(err))}
    print("sequential_fp64", json.dumps(res["sequential_fp64"]), flush=True)
    print("cd", json.dumps({k: v for k, v in res["cd"].items() if "err" in k}), flush=True)
    if out_path:
        with open(out_path, "w") as fh:
            json.dump(res, fh, indent=1)
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("study", choices=["precision", "adjoint", "batch"])
    ap.add_argument("--case", choices=["sphere", "channel2d"], default="sphere",
                    help="precision: the D3Q27 sphere box or the D2Q9 400x100 channel")
    ap.add_argument("--seed", type=int, default=1234, help="precision: perturbation seed")
    ap.add_argument("--layout", choices=["rows", "soa"], default=None,
                    help="precision: population layout (default: the solver's)")
    ap.add_argument("--nx", type=int, default=768)
    ap.add_argument("--ny", type=int, default=384)
    ap.add_argument("--nz", type=int, default=384)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--window", type=int, default=5000)
    ap.add_argument("--peak", type=float, default=None,
                    help="HBM peak in GB/s (default: MEASURED_PEAKS.json)")
    ap.add_argument("--out", default=None)
    ap.add_argument("--forms", default=",".join(f[0] for f in FORMS))
    ap.add_argument("--directions", type=int, default=16)
    ap.add_argument("--checkpoint", type=int, default=100)
    ap.add_argument("--precisions", default="fp32,fp64")
    ap.add_argument("--no-fd", action="store_true")
    ap.add_argument("--instances", type=int, default=64)
    ap.add_argument("--no-sequential", action="store_true",
                    help="batch: skip the one-at-a-time FP64 comparison")
    ap.add_argument("--shape", default=None,
                    help="batch: fixed launch shape 'tile_height,blocks_per_sm' instead of "
                         "autotuning (blocks_per_sm 0: one interior item per block)")
    args = ap.parse_args()
    if args.peak is None:
        args.peak = measured_peak_gbs()
    if args.study == "batch":
        steps = args.steps
        shape = tuple(int(v) for v in args.shape.split(",")) if args.shape else None
        batch_study(args.instances, steps, window=steps // 2, peak_gbs=args.peak,
                    out_path=args.out, sequential=not args.no_sequential, shape=shape)
        return
    if args.study == "adjoint":
        steps = args.steps if args.steps != 20000 else 7000
        window = (steps - 2000, steps) if steps > 2000 else (steps // 2, steps)
        nx = args.nx if args.nx != 768 else 1024
        ny = args.ny if args.ny != 384 else 256
        adjoint_study(steps, window, args.checkpoint, directions=args.directions,
                      out_path=args.out, nx=nx, ny=ny,
                      precisions=tuple(args.precisions.split(",")), fd=not args.no_fd)
        return
    keep = set(args.forms.split(","))
    forms = [f for f in FORMS if f[0] in keep]
    if args.case == "channel2d":
        case = channel2d_case(seed=args.seed)
    else:
        case = sphere_case(args.nx, args.ny, args.nz, diam=64.0 * args.nx / 768.0,
                           seed=args.seed)
    if args.layout:
        case["layout"] = args.layout
    precision_study(case, args.steps, args.window, args.peak, forms, args.out)


if __name__ == "__main__":
    main()
