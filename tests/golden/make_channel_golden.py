"""Oracle fixtures for the benchmark channel problem (no reference counterpart).

The reference hard-codes its own boundaries and geometry, so the benchmark
channel problems are pinned to the CPU oracle (oracle/lbm_oracle.cpp, itself
pinned bit-for-bit to the reference's sources on the shared physics).  This
script runs the oracle on the small 2-D benchmark problem -- D2Q9 400x100,
cylinder D = 20 at (80, 50), u_in = 0.05, Re = 100, free-slip walls, seeded
+-1e-3 u_y perturbation, 20,000 steps -- and stores the per-step force of the
first 3,000 steps plus Cd mean, Cl rms and St over the last 10,000 steps.  The
shedding of this problem still grows until about step 28,000, so the same
statistics are also stored for steps 30,000-40,000 of a 40,000-step run
(`stats_periodic`), where the flow is periodic.

    python tests/golden/make_channel_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "cylinder-flow_gb300"))

from oracle import oracle as O  # noqa: E402

CASE = dict(lattice=9, nx=400, ny=100, tau0=3 * 0.05 * 20 / 100, u0=0.05, wall_y="freeslip",
            geom="cylinder", cx=80.0, cy=50.0, diam=20.0, perturb_amp=1e-3, seed=1234)
STEPS, WINDOW, KEEP = 20000, 10000, 3000
STEPS_PERIODIC = 40000


def main() -> None:
    from cflbm import analysis
    c = O.channel_cfg(9, CASE["nx"], CASE["ny"], tau0=CASE["tau0"], u_in=CASE["u0"],
                      wall_y=O.WALL_FREESLIP, geom=O.GEOM_CYLINDER, cx=CASE["cx"],
                      cy=CASE["cy"], diam=CASE["diam"], amp=CASE["perturb_amp"],
                      seed=CASE["seed"])
    o = O.channel(c, STEPS, want_f=False)
    stats = analysis.summary(o["force"], CASE["u0"], CASE["diam"], CASE["diam"], WINDOW)
    o2 = O.channel(c, STEPS_PERIODIC, want_f=False)
    assert np.array_equal(o2["force"][:STEPS], o["force"])
    stats_periodic = analysis.summary(o2["force"], CASE["u0"], CASE["diam"], CASE["diam"],
                                      WINDOW)
    np.savez_compressed(os.path.join(HERE, "channel_d2q9_400x100.npz"),
                        meta=json.dumps(dict(case=CASE, steps=STEPS, window=WINDOW, stats=stats,
                                             steps_periodic=STEPS_PERIODIC,
                                             stats_periodic=stats_periodic)),
                        force=o["force"][:KEEP, :2], u=o["u"][0], v=o["v"][0])
    print(stats)
    print(stats_periodic)


if __name__ == "__main__":
    main()
