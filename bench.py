"""Benchmark of the hot path: MLUPS and the HBM roofline of the fused LBM sweep.

Workload (default): D3Q27 BGK flow past a spanwise cylinder on a 512x128x128
grid (D = 32 cells, axis along z through (128, 64)), equilibrium inlet
u = (0.04, 0, 0), zero-gradient outlet, free-slip y, periodic z, Re = 200
(tau = 0.5 + 3 u D / Re = 0.5192), initial rho = 1, uniform u plus a seeded
+-1e-3 u_y perturbation.  The headline stores FP64 populations and computes in
FP64, the reference's arithmetic (GB300's FP64 units run at ~1.2 TFLOP/s, so
this form is bound by them, not by HBM).  The other forms -- double-float
collision on FP64 storage, FP32 collision on FP64 / FP32 storage, FP16
deviation storage, both layouts -- are measured on the same grid under `forms`,
each with its error after a few steps against the FP64 oracle's run of the
same steps.

One step = one time step of the whole grid (fused sweep + the body-force
launch beside it).  `value` = interior cells x timed steps / device time
(MLUPS), inputs resident; the sweep time of the same steps comes from events
around every sweep launch on the solver's stream; `e2e` = the same metric
through the C ABI end to end: create the handle from host buffers (page-locked
solid mask), step, read every step's force back to page-locked host memory as
the reference's test.dat loop does (queued behind the step, so the next step is
queued before it arrives), and read the final u, v, w, p fields back.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

`--impl reference` times the FP64 oracle's run of the same workload on all
host cores (W warm-up and K timed steps, capped at 5 and 20).
`--workload channel2d` measures the small D2Q9 400x100 channel instead, over its
whole 20,000-step run, in every storage form, with the run's Cd, Cl and St.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "cylinder-flow_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

NX, NY, NZ = 512, 128, 128
D, U_IN, RE = 32.0, 0.04, 200.0
TAU0 = 3.0 * U_IN * D / RE           # reference System::tau; tau = tau0 + 0.5
WORKLOAD = dict(lattice=27, nx=NX, ny=NY, nz=NZ, tau0=TAU0, u0=U_IN, wall_y="freeslip",
                wall_z="periodic", geom="cylinder", cx=128.0, cy=64.0, diam=D,
                perturb_amp=1e-3, seed=1234)
CELLS = NX * NY * NZ
ERR_STEPS = 3  # steps of the forms' error check against the oracle
METRIC = "MLUPS (D3Q27 BGK sweep, 512x128x128 spanwise cylinder)"


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            m = json.load(fh)
        return float(m["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(name="sweep_fp64_d3q27_512x128x128.md"):
    """Per-launch DRAM bytes of the headline sweep (FP64 storage and arithmetic)
    from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._proc = None

    def __enter__(self):
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self._proc = None
        return self

    def _read(self):
        for line in self._proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 8:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4)
                          if r[4 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        import torch
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    from cflbm.replicas import max_over_ranks as _m
    return _m(x, world)


def timed_steps(solver, steps, stream):
    """Device time of `steps` steps (CUDA events on the solver's stream around
    the whole region) and the per-step sweep time of the same steps (events the
    library records around every sweep launch on that stream)."""
    import torch
    solver.set_timing(True)
    solver.timing()  # reset
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    solver.step(steps)
    e1.record(stream)
    e1.synchronize()
    sw_ms, _, n_sw, _ = solver.timing()
    solver.set_timing(False)
    return e0.elapsed_time(e1), sw_ms / max(n_sw, 1)


def form_errors(s, oracle_run):
    """Errors of a solver's state after ERR_STEPS steps from t = 0 against the
    FP64 oracle's run of the same steps: relative L-inf of u, v, w, p and of the
    last step's drag force."""
    u, v, w, p = s.macros()
    fh = s.force_history()
    o = oracle_run
    rel = lambda a, b: float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))  # noqa: E731
    return {"steps": ERR_STEPS, "u": rel(u, o["u"]), "v": rel(v, o["v"]), "w": rel(w, o["w"]),
            "p": rel(p, o["p"]), "fx": abs(fh[-1, 0] - o["force"][-1, 0]) / abs(o["force"][-1, 0])}


def variant(cflbm, local, storage, compute, layout, steps, warmup, oracle_run,
            rounding="stochastic"):
    import torch
    with cflbm.Solver(device=local, storage=storage, compute=compute, layout=layout,
                      rounding=rounding, **WORKLOAD) as s:
        err = None
        if oracle_run is not None:
            s.step(ERR_STEPS)
            err = form_errors(s, oracle_run)
        stream = torch.cuda.ExternalStream(s.stream_ptr())
        s.step(warmup)
        s.synchronize()
        ms, sweep_ms = timed_steps(s, steps, stream)
        info = s.info()
    out = {"mlups": CELLS * steps / (ms * 1e-3) / 1e6, "ms_per_step": ms / steps,
           "sweep_us": 1e3 * sweep_ms, "bytes_per_cell": info.bytes_per_cell_step}
    if err is not None:
        out["error_vs_oracle"] = err
    return out


def oracle_cfg():
    from oracle import oracle as O
    return O.channel_cfg(27, NX, NY, NZ, tau0=TAU0, u_in=U_IN, wall_y=O.WALL_FREESLIP,
                         wall_z=O.WALL_PERIODIC, geom=O.GEOM_CYLINDER, cx=128.0, cy=64.0,
                         diam=D, amp=1e-3, seed=1234)


def run_gb300(args):
    world, rank, local = dist_setup(args)
    import torch
    import cflbm

    peak, peak_kind = peaks()
    steps, warmup = args.steps, args.warmup
    # ---- CPU: the FP64 oracle on the same workload (the reference's algorithm
    # with the workload's boundaries), a bounded number of steps: the CPU
    # baseline, and the reference every form's error is stated against ----------
    cpu, oracle_run = None, None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu, oracle_run = cpu_baseline(args.cpu_steps)

    # ---- device-resident timing of the headline: FP64 storage, FP64 arithmetic --
    with cflbm.Solver(device=local, storage="fp64", compute="fp64", **WORKLOAD) as s:
        err64 = None
        if oracle_run is not None:
            s.step(ERR_STEPS)
            err64 = form_errors(s, oracle_run)
        stream = torch.cuda.ExternalStream(s.stream_ptr())
        s.step(warmup)
        s.synchronize()
        barrier(world)
        torch.cuda.synchronize()
        with ClockSampler(local) as clk:
            s.step(warmup)  # keep the GPU busy while the sampler starts
            time.sleep(0.3)
            s.synchronize()
            n_launch0 = cflbm.launch_count()
            ms, sweep_ms = timed_steps(s, steps, stream)
            n_launch = cflbm.launch_count() - n_launch0
        torch.cuda.synchronize()
        barrier(world)
        ms = max_over_ranks(ms, world)
        info = s.info()
        f, cdcl = s.forces()
        mass, _ = s.mass()
    value = world * CELLS * steps / (ms * 1e-3) / 1e6
    sweep_s = sweep_ms * 1e-3
    achieved = info.bytes_per_cell_step * CELLS / sweep_s / 1e9
    traffic = profile_traffic()

    # ---- the other storage/arithmetic forms at the same grid ---------------------
    extra = {}
    if not args.quick:
        for name, st, cp, lay in (("df64_arith", "fp64", "df64", "rows"),
                                  ("fp32_collision", "fp64", "fp32", "rows"),
                                  ("fp32_collision_soa", "fp64", "fp32", "soa"),
                                  ("fp32_store", "fp32", "fp32", "rows"),
                                  ("fp32_store_soa", "fp32", "fp32", "soa"),
                                  ("fp16dev_store", "fp16dev", "fp32", "rows"),
                                  ("fp16dev_store_soa", "fp16dev", "fp32", "soa"),
                                  ("fp16dev_rn_store_soa", "fp16dev", "fp32", "soa")):
            v = variant(cflbm, local, st, cp, lay, steps, min(warmup, 5), oracle_run,
                        "nearest" if "_rn_" in name else "stochastic")
            v["hbm_frac"] = v["bytes_per_cell"] * CELLS / (v["sweep_us"] * 1e-6) / 1e9 / peak
            extra[name] = {k: (round(x, 4) if isinstance(x, float) else x) for k, x in v.items()}

    # ---- end to end through the C ABI with host buffers --------------------------
    e2e_steps = max(steps, 10)  # as many steps as the device-timed leg
    solid = np.zeros((NZ, NY, NX), np.uint8)
    yy, xx = np.mgrid[0:NY, 0:NX]
    solid[:, ((xx - 128.0) ** 2 + (yy - 64.0) ** 2) <= (D / 2) ** 2] = 1
    solid_pinned = torch.from_numpy(solid).pin_memory()
    pinned = [torch.empty((NZ, NY, NX), dtype=torch.float64).pin_memory() for _ in range(4)]
    forces_pinned = torch.zeros((e2e_steps, 3), dtype=torch.float64).pin_memory()
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    wl = dict(WORKLOAD)
    wl["geom"] = "none"
    with cflbm.Solver(device=local, storage="fp64", compute="fp64", solid=solid_pinned.numpy(),
                      **wl) as s:
        t_created = time.perf_counter()
        for k in range(e2e_steps):
            s.step(1)
            # every step's force read back to the host (the reference writes
            # Cd/Cl to test.dat every step), queued behind the step
            s.forces_async(forces_pinned[k].data_ptr())
        outs = [t.numpy() for t in pinned]
        cflbm._lib.check(cflbm._lib.lib.cflbm_macros(
            s._h, *[o.ctypes.data_as(cflbm.solver.ctypes.POINTER(cflbm.solver.ctypes.c_double))
                    for o in outs]), "cflbm_macros")  # synchronises
        hist_last = s.force_history()[-1]
    t1 = time.perf_counter()
    forces_ok = bool(np.array_equal(forces_pinned[-1].numpy(), hist_last))
    e2e_s = max_over_ranks(t1 - t0, world)
    e2e_value = world * CELLS * e2e_steps / e2e_s / 1e6
    h2d = solid.nbytes / e2e_steps
    d2h = (e2e_steps * 3 * 8 + 4 * CELLS * 8) / e2e_steps

    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "MLUPS", "n_gpus": world,
        "steps": steps, "warmup": warmup, "ms_per_step": round(ms / steps, 5),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded perturbation; no dataset)",
        "config": {"workload": "D3Q27 512x128x128 spanwise cylinder D=32, Re=200, "
                               "free-slip y, periodic z",
                   "storage": "f64", "collision": "f64", "global_cells": CELLS * world,
                   "parallelism": f"replicas x{world}",
                   "l2": "working set 2 x 3.8 GB >> 129 MB L2 (no flush needed)"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "traffic": traffic, "peak_source": peak_kind,
                     "bytes_per_cell": info.bytes_per_cell_step,
                     "sweep_us": round(sweep_s * 1e6, 2),
                     "note": "FP64 arithmetic is bound by GB300's FP64 units, not HBM: "
                             "133 FP64 instructions per cell at 85 % FP64-pipe activity "
                             "(ncu, profiles/sweep_instruction_mix_d3q27.md)"},
        "e2e": {"value": round(e2e_value, 2), "unit": "MLUPS", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "steps": e2e_steps, "forces_read_back": forces_ok,
                "create_ms": round(1e3 * (t_created - t0), 2)},
        "gpu_launches": n_launch,
        "clocks": clk.summary(),
        "error_vs_oracle": err64,
        "forms": extra,
        "check": {"cd": cdcl[0], "cl": cdcl[1], "mass": mass, "finite": bool(np.isfinite(mass))},
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


# ---- the small channel problem: D2Q9 400x100 cylinder, 20,000 steps ---------------
# Cylinder D = 20 at (80, 50), equilibrium inlet u = (0.05, 0), zero-gradient
# outlet, free-slip walls, Re = 100 (tau = 0.5 + 3 u D / Re), seeded +-1e-3 u_y
# perturbation; Cd, Cl and St over the last 10,000 steps.  40,000 cells: the
# whole state (2 x 2.9 MB in FP64) stays in L2, so a step is bound by launch and
# latency, not by HBM.
CH2D = dict(lattice=9, nx=400, ny=100, tau0=3 * 0.05 * 20 / 100, u0=0.05, wall_y="freeslip",
            geom="cylinder", cx=80.0, cy=50.0, diam=20.0, perturb_amp=1e-3, seed=1234)
CH2D_CELLS = 400 * 100
CH2D_WINDOW = 10000
METRIC_2D = "MLUPS (D2Q9 BGK sweep, 400x100 cylinder channel, 20,000-step run)"


def run_channel2d(args):
    """Every storage/arithmetic form over the full 20,000-step run, device time
    from t = 0 (the warm-up steps run first and the state is then reset to the
    initial one), the run's Cd mean, Cl rms and St, and the plain FP64 form end
    to end from host buffers."""
    world, rank, local = dist_setup(args)
    import torch
    import cflbm
    from cflbm import analysis

    peak, peak_kind = peaks()
    steps, warmup = args.steps, args.warmup
    forms = {}
    n_launch = 0
    with ClockSampler(local) as clk:
        for name, st, cp in (("fp64", "fp64", "fp64"), ("df64", "fp64", "df64"),
                             ("fp64_store", "fp64", "fp32"), ("fp32_store", "fp32", "fp32"),
                             ("fp16dev_store", "fp16dev", "fp32"),
                             ("fp16dev_rn_store", "fp16dev", "fp32")):
            with cflbm.Solver(device=local, storage=st, compute=cp, force_history=steps + 8,
                              rounding="nearest" if "_rn_" in name else "stochastic",
                              **CH2D) as s:
                stream = torch.cuda.ExternalStream(s.stream_ptr())
                f0 = s.get_f()
                s.step(warmup)
                s.set_f(f0, 0)
                s.synchronize()
                barrier(world)
                torch.cuda.synchronize()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                l0 = cflbm.launch_count()
                e0.record(stream)
                s.step(steps)
                e1.record(stream)
                e1.synchronize()
                launches = cflbm.launch_count() - l0
                ms = max_over_ranks(e0.elapsed_time(e1), world)
                hist = s.force_history(steps)
                stats = analysis.summary(hist, CH2D["u0"], CH2D["diam"], CH2D["diam"],
                                         min(CH2D_WINDOW, steps))
                info = s.info()
            if name == "fp64":
                n_launch = launches
            forms[name] = {"mlups": round(world * CH2D_CELLS * steps / (ms * 1e-3) / 1e6, 2),
                           "us_per_step": round(1e3 * ms / steps, 3),
                           "bytes_per_cell": info.bytes_per_cell_step,
                           "cd_mean": stats["cd_mean"],
                           "cd_mean_periods": stats["cd_mean_periods"],
                           "periods": stats["periods"], "cl_rms": stats["cl_rms"],
                           "st": stats["st"]}
    ref = forms["fp64"]
    for v in forms.values():
        v["cd_rel_err"] = abs(v["cd_mean"] - ref["cd_mean"]) / abs(ref["cd_mean"])
        v["cd_periods_rel_err"] = (abs(v["cd_mean_periods"] - ref["cd_mean_periods"])
                                   / abs(ref["cd_mean_periods"]))
        v["st_rel_err"] = abs(v["st"] - ref["st"]) / abs(ref["st"]) if ref["st"] else None

    # ---- end to end, plain FP64 form: solid mask from the host, the run, the
    # force history and the final u, v, w, p fields back to the host --------------
    solid = np.zeros((1, CH2D["ny"], CH2D["nx"]), np.uint8)
    yy, xx = np.mgrid[0:CH2D["ny"], 0:CH2D["nx"]]
    solid[0, ((xx - CH2D["cx"]) ** 2 + (yy - CH2D["cy"]) ** 2) <= (CH2D["diam"] / 2) ** 2] = 1
    wl = dict(CH2D)
    wl["geom"] = "none"
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    with cflbm.Solver(device=local, storage="fp64", compute="fp64", solid=solid,
                      force_history=steps + 8, **wl) as s:
        s.step(steps)
        hist = s.force_history(steps)
        u, v, w, p = s.macros()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    e2e = {"value": round(world * CH2D_CELLS * steps / e2e_s / 1e6, 2), "unit": "MLUPS",
           "h2d_bytes_per_step": solid.nbytes / steps,
           "d2h_bytes_per_step": (hist.nbytes + u.nbytes + v.nbytes + w.nbytes + p.nbytes) / steps,
           "steps": steps}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline_2d(args.cpu_steps_2d)
    bpc = ref["bytes_per_cell"]
    achieved = bpc * CH2D_CELLS / (ref["us_per_step"] * 1e-6) / 1e9
    line = {
        "metric": METRIC_2D, "value": ref["mlups"], "unit": "MLUPS", "n_gpus": world,
        "steps": steps, "warmup": warmup, "ms_per_step": round(ref["us_per_step"] / 1e3, 6),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded perturbation; no dataset)",
        "config": {"workload": "D2Q9 400x100 cylinder channel D=20, Re=100, free-slip walls, "
                               "20,000 steps",
                   "storage": "f64", "collision": "f64", "global_cells": CH2D_CELLS * world,
                   "parallelism": f"replicas x{world}",
                   "l2": "working set 2 x 2.9 MB, L2-resident (the problem's own size)"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": None,
                     "peak_source": peak_kind, "bytes_per_cell": bpc,
                     "note": "L2-resident and launch-bound: two launches per step"},
        "e2e": e2e, "gpu_launches": n_launch, "clocks": clk.summary(), "forms": forms,
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def cfg_2d():
    from oracle import oracle as O
    return O.channel_cfg(9, CH2D["nx"], CH2D["ny"], tau0=CH2D["tau0"], u_in=CH2D["u0"],
                         wall_y=O.WALL_FREESLIP, geom=O.GEOM_CYLINDER, cx=CH2D["cx"],
                         cy=CH2D["cy"], diam=CH2D["diam"], amp=1e-3, seed=1234)


def cpu_baseline_2d(steps: int):
    """The small channel on the host cores: the FP64 oracle's channel run (the
    reference's passes with this problem's boundaries), OpenMP over all cores,
    timed per step over a bounded number of steps."""
    from oracle import oracle as O
    cores = os.cpu_count() or 1
    o = O.channel(cfg_2d(), steps, nthreads=cores, want_f=False)
    t = float(np.sum(o["step_seconds"]))
    return {"value": round(CH2D_CELLS * steps / max(t, 1e-9) / 1e6, 3), "unit": "MLUPS",
            "cores": cores, "kind": "port",
            "sample": f"{steps} of the 20,000 steps of the 400x100 D2Q9 channel (oracle port of "
                      f"the reference solver's passes, FP64), initialisation excluded"}


def cpu_baseline(steps: int):
    """The workload on the host cores: the FP64 oracle's channel run (the
    reference's collide / stream / update passes with the workload's
    boundaries), OpenMP over all cores, timed per step (initialisation
    excluded) over a bounded number of steps.  Returns the baseline record and
    the run's fields and forces, the reference of the forms' errors."""
    from oracle import oracle as O
    cores = os.cpu_count() or 1
    o = O.channel(oracle_cfg(), steps, nthreads=cores, want_f=False)
    t_run = float(np.sum(o["step_seconds"]))
    rec = {"value": round(CELLS * steps / max(t_run, 1e-9) / 1e6, 3), "unit": "MLUPS",
           "cores": cores, "kind": "port",
           "sample": f"{steps} steps of the 512x128x128 D3Q27 workload (oracle port of the "
                     f"reference solver's passes, FP64), initialisation excluded"}
    return rec, o


def run_reference(args):
    """The reference's algorithm on the host cores, on this arm's workload and
    metric: the FP64 oracle port (the compiled reference cannot run here: its
    sources are not on this machine and it hard-codes its own geometry and
    boundaries).  W warm-up steps then K timed steps in one run, each step timed
    on the host clock; K and W are capped (20 and 5) so the run stays within a
    few minutes."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from oracle import oracle as O
    two_d = args.workload == "channel2d"
    steps, warmup = min(args.steps, 20), min(args.warmup, 5)
    cores = os.cpu_count() or 1
    if two_d:
        cfg = cfg_2d()
        cells = CH2D_CELLS
        steps, warmup = args.steps, args.warmup  # the small grid runs every step
    else:
        cfg = oracle_cfg()
        cells = CELLS
    o = O.channel(cfg, warmup + steps, nthreads=cores, want_f=False)
    t = float(np.sum(o["step_seconds"][warmup:]))
    v = round(cells * steps / max(t, 1e-9) / 1e6, 3)
    line = {
        "metric": METRIC_2D if two_d else METRIC, "value": v, "unit": "MLUPS", "n_gpus": world,
        "steps": steps, "warmup": warmup, "ms_per_step": round(1e3 * t / steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded perturbation; no dataset)",
        "impl": "reference",
        "config": {"workload": (
            "D2Q9 400x100 cylinder channel D=20, Re=100, free-slip walls" if two_d else
            "D3Q27 512x128x128 spanwise cylinder D=32, Re=200, free-slip y, periodic z"),
            "storage": "f64", "collision": "f64", "global_cells": cells},
        "cpu_baseline": {"value": v, "unit": "MLUPS", "cores": cores, "kind": "port",
                         "sample": f"{steps} timed steps after {warmup} warm-up steps of the "
                                   f"workload (oracle port of the reference solver's passes, "
                                   f"FP64, OpenMP on all host cores)"},
        "e2e": {"value": v, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_profile(args):
    """A bare stepping loop for profiler captures (no extras, no CPU baseline).
    --ref: the reference-rule D3Q27 profile (the reference's face passes, sphere
    and solid rule) on the same grid instead of the channel problem."""
    import cflbm
    if args.ref:
        wl = dict(lattice=27, nx=args.nx, ny=args.ny, nz=args.nz, profile="ref3d", tau0=TAU0,
                  u0=U_IN)
    else:
        wl = dict(WORKLOAD, nx=args.nx, ny=args.ny, nz=args.nz, cx=args.nx / 4.0,
                  cy=args.ny / 2.0)
    for layout in args.layout.split(","):  # one layout after the other
        with cflbm.Solver(storage=args.storage, compute=args.compute, layout=layout,
                          rounding=args.rounding, **wl) as s:
            s.step(args.warmup)
            s.synchronize()
            t0 = time.perf_counter()
            s.step(args.steps)
            s.synchronize()
            dt = time.perf_counter() - t0
            info = s.info()
        cells = args.nx * args.ny * args.nz
        print(json.dumps({"profile_case": [args.nx, args.ny, args.nz],
                          "profile": "ref3d" if args.ref else "channel",
                          "storage": args.storage, "compute": args.compute, "layout": layout,
                          "rounding": args.rounding, "steps": args.steps,
                          "mlups_wall": cells * args.steps / dt / 1e6,
                          "bytes_per_cell": info.bytes_per_cell_step,
                          "device_bytes": info.device_bytes}))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--workload", default="cylinder3d", choices=["cylinder3d", "channel2d"],
                    help="cylinder3d: D3Q27 512x128x128 (the benchmark line); channel2d: "
                         "D2Q9 400x100 over its 20,000-step run")
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 1000; 20000 for channel2d)")
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--quick", action="store_true", help="headline variant only")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--cpu-steps-2d", type=int, default=4000)
    ap.add_argument("--profile", action="store_true",
                    help="bare stepping loop on an --nx/--ny/--nz grid for profiler captures")
    ap.add_argument("--ref", action="store_true",
                    help="with --profile: the reference-rule D3Q27 profile")
    ap.add_argument("--nx", type=int, default=NX)
    ap.add_argument("--ny", type=int, default=NY)
    ap.add_argument("--nz", type=int, default=NZ)
    ap.add_argument("--storage", default="fp64", choices=["fp64", "fp32", "fp16dev"])
    ap.add_argument("--compute", default="fp32", choices=["fp64", "fp32", "df64"])
    ap.add_argument("--layout", default="rows",
                    help="soa or rows; with --profile a comma list runs each in turn")
    ap.add_argument("--rounding", default="stochastic", choices=["nearest", "stochastic"],
                    help="FP16 storage rounding (with --profile)")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 20000 if args.workload == "channel2d" else 1000
    if args.warmup < 3:
        args.warmup = 3
    if args.profile:
        return run_profile(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "channel2d":
        return run_channel2d(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
