"""The small benchmark problem at full length on the GPU: D2Q9 400x100 cylinder
channel, 20,000 steps, against the oracle's fixture (tests/golden/
make_channel_golden.py).  Early forces are compared step by step; the drag
averaged over the whole shedding periods of the last 10,000 steps, the lift rms
and St are compared as statistics, since vortex shedding amplifies round-off
differences in the phase."""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

import cflbm
from cflbm import Solver, analysis

pytestmark = pytest.mark.gpu


def fixture():
    z = np.load(os.path.join(GOLDEN, "channel_d2q9_400x100.npz"))
    meta = json.loads(str(z["meta"]))
    return meta, z["force"], z["u"], z["v"]


# tol_stats bounds the relative error of the drag averaged over whole shedding
# periods (analysis.summary's cd_mean_periods) and of St; the lift rms gets 5x.
# FP16 deviation storage is held to the 1e-3 drag bar of the precision form.
@pytest.mark.parametrize("storage,compute,tol_f,tol_stats", [
    ("fp64", "fp64", 1e-9, 1e-3),
    ("fp64", "df64", 1e-9, 1e-3),
    ("fp64", "fp32", 1e-4, 1e-3),
    ("fp32", "fp32", 1e-4, 1e-3),
    ("fp16dev", "fp32", 5e-2, 1e-3),
])
def test_config1_statistics_match_oracle(cuda, storage, compute, tol_f, tol_stats):
    meta, force, _, _ = fixture()
    case = meta["case"]
    with Solver(storage=storage, compute=compute, force_history=meta["steps"] + 8, **case) as s:
        s.step(meta["steps"])
        hist = s.force_history(meta["steps"])
    k = min(1000, force.shape[0])
    scale = np.max(np.abs(force[:k, 0]))
    assert np.max(np.abs(hist[:k, 0] - force[:k, 0])) <= tol_f * scale
    st = analysis.summary(hist, case["u0"], case["diam"], case["diam"], meta["window"])
    ref = meta["stats"]
    assert st["periods"] >= 3 and ref["periods"] >= 3
    assert abs(st["cd_mean_periods"] - ref["cd_mean_periods"]) <= tol_stats * abs(
        ref["cd_mean_periods"])
    # the lift rms: 5x the drag bar; FP16 storage 2e-2 (its rounding noise adds
    # lift fluctuations)
    tol_cl = 2e-2 if storage == "fp16dev" else 5 * tol_stats
    assert abs(st["cl_rms"] - ref["cl_rms"]) <= tol_cl * abs(ref["cl_rms"])
    assert abs(st["st"] - ref["st"]) <= tol_stats * abs(ref["st"])
