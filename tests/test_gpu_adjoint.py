"""The hand-written adjoint (cflbm_adjoint) against central finite differences.

J = mean drag over a step window of a D2Q9 cylinder channel with a Brinkman
porosity field around the body.  Gradients with respect to the inlet speed,
tau and the porosity field (along 16 seeded directions) are compared with
central differences at h = 1e-4 of the FP64 GPU solver and of the CPU oracle,
the FP32 adjoint with the FP64 one, and checkpoint spacings with each other.

Tolerances: FP64 adjoint vs FP64 finite differences 1e-5 relative for the
scalars; 1e-4 relative (no absolute floor) along every porosity direction,
against the Richardson extrapolation of differences at h and 2h; FP32 adjoint vs
FP64 adjoint 1e-2 relative (FP32 round-off accumulated over the run).
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O

import cflbm
from cflbm import Solver
from cflbm.adjoint import drag_objective, run, smooth_porosity

pytestmark = pytest.mark.gpu

H = 1e-4
STEPS, K, WINDOW = 300, 40, (150, 300)
BASE = dict(lattice=9, nx=96, ny=48, geom="cylinder", cx=30, cy=24, diam=10,
            perturb_amp=1e-3, seed=1234)
U_IN = 0.05
TAU = 0.5 + 3 * U_IN * 10 / 20  # Re = 20
WALLS = ["freeslip", "noslip", "periodic"]


def case(wall="freeslip", prec="fp64"):
    c = dict(BASE, wall_y=wall)
    c["storage"] = c["compute"] = prec
    return c


def alpha_field():
    """Porosity in [0, 0.3] on a box around the cylinder, rounded to FP32 (the
    solver stores alpha in FP32)."""
    a = 0.3 * smooth_porosity(96, 48, (14, 8, 46, 40), seed=7)
    return a.astype(np.float32).astype(np.float64)


def J_gpu(c, alpha, u_in, tau, steps=STEPS, window=WINDOW):
    with Solver(**c, u0=u_in, tau0=tau - 0.5, alpha=alpha, force_history=steps) as s:
        s.step(steps)
        f = s.force_history(steps)
    return float(np.mean(f[window[0] - 1:window[1], 0]))


def J_oracle(wall, alpha, u_in, tau, steps=STEPS, window=WINDOW):
    w = {"freeslip": O.WALL_FREESLIP, "noslip": O.WALL_NOSLIP, "periodic": O.WALL_PERIODIC}
    cfg = O.channel_cfg(9, 96, 48, tau0=tau - 0.5, u_in=u_in, wall_y=w[wall],
                        geom=O.GEOM_CYLINDER, cx=30, cy=24, diam=10, amp=1e-3, seed=1234,
                        alpha=alpha)
    f = O.channel(cfg, steps, want_f=False)["force"]
    return float(np.mean(f[window[0] - 1:window[1], 0]))


_CACHE = {}


def adj(wall="freeslip", prec="fp64", k=K):
    key = (wall, prec, k)
    if key not in _CACHE:
        _CACHE[key] = run(case(wall, prec), alpha_field(), U_IN, TAU, STEPS, k, WINDOW)
    return _CACHE[key]


@pytest.mark.parametrize("wall", WALLS)
def test_adjoint_scalars_match_finite_differences(cuda, wall):
    r = adj(wall)
    a = alpha_field()
    c = case(wall)
    assert abs(r["J"] - J_gpu(c, a, U_IN, TAU)) <= 1e-13 * abs(r["J"])
    fd_u = (J_gpu(c, a, U_IN + H, TAU) - J_gpu(c, a, U_IN - H, TAU)) / (2 * H)
    fd_t = (J_gpu(c, a, U_IN, TAU + H) - J_gpu(c, a, U_IN, TAU - H)) / (2 * H)
    assert abs(r["dJ_du_in"] - fd_u) <= 1e-5 * abs(fd_u), (r["dJ_du_in"], fd_u)
    assert abs(r["dJ_dtau"] - fd_t) <= 1e-5 * abs(fd_t), (r["dJ_dtau"], fd_t)


def test_adjoint_porosity_gradient_along_16_directions(cuda):
    """Relative error of the projection dJ/dalpha . d along 16 seeded random
    directions, each against central differences at h and 2h combined by
    Richardson extrapolation, (4 D(h) - D(2h)) / 3, which removes the
    differences' h^2 truncation term: a direction whose projection is small
    next to J's third derivative along it would otherwise read that term as
    adjoint error."""
    r = adj()
    g = r["dJ_dalpha"]
    a = alpha_field()
    c = case()
    rng = np.random.default_rng(2024)
    box = np.zeros_like(a)
    box[8:40, 14:46] = 1.0
    errs = []
    for _ in range(16):
        d = rng.standard_normal(a.shape) * box
        d /= np.max(np.abs(d))
        fd, ad = [], []
        for h in (H, 2 * H):
            ap = (a + h * d).astype(np.float32).astype(np.float64)
            am = (a - h * d).astype(np.float32).astype(np.float64)
            fd.append((J_gpu(c, ap, U_IN, TAU) - J_gpu(c, am, U_IN, TAU)) / (2 * h))
            ad.append(float(np.sum(g * (ap - am))) / (2 * h))
        fr = (4 * fd[0] - fd[1]) / 3
        ar = (4 * ad[0] - ad[1]) / 3
        errs.append(abs(ar - fr) / abs(fr))
    assert max(errs) <= 1e-4, errs


def test_adjoint_matches_oracle_finite_differences(cuda):
    """An FP64 reference gradient independent of the GPU code: central
    differences of the CPU oracle."""
    r = adj()
    a = alpha_field()
    assert abs(r["J"] - J_oracle("freeslip", a, U_IN, TAU)) <= 1e-10 * abs(r["J"])
    fd_u = (J_oracle("freeslip", a, U_IN + H, TAU) - J_oracle("freeslip", a, U_IN - H, TAU)) / (2 * H)
    assert abs(r["dJ_du_in"] - fd_u) <= 1e-5 * abs(fd_u)
    d = np.zeros_like(a)
    d[20:30, 22:40] = 1.0  # the porous band upstream and around the body
    fd_a = (J_oracle("freeslip", a + H * d, U_IN, TAU) -
            J_oracle("freeslip", a - H * d, U_IN, TAU)) / (2 * H)
    ad_a = float(np.sum(r["dJ_dalpha"] * d))
    assert abs(ad_a - fd_a) <= 1e-5 * abs(fd_a), (ad_a, fd_a)


def test_checkpoint_spacing_does_not_change_the_gradient(cuda):
    """K = 1, 7 (odd, not a divisor), 150 (two segments), the run length (one
    segment) against K = 40: every schedule of the segment pipeline."""
    r2 = adj(k=K)
    for r in (adj(k=1), adj(k=7), adj(k=150), adj(k=STEPS)):
        assert r["J"] == r2["J"]
        assert r["dJ_du_in"] == r2["dJ_du_in"]
        assert r["dJ_dtau"] == r2["dJ_dtau"]
        assert np.max(np.abs(r["dJ_dalpha"] - r2["dJ_dalpha"])) <= 1e-12 * np.max(
            np.abs(r2["dJ_dalpha"]))


def test_fp32_adjoint_against_fp64_reference_gradient(cuda):
    r64, r32 = adj(), adj(prec="fp32")
    assert abs(r32["J"] - r64["J"]) <= 1e-4 * abs(r64["J"])
    assert abs(r32["dJ_du_in"] - r64["dJ_du_in"]) <= 1e-2 * abs(r64["dJ_du_in"])
    assert abs(r32["dJ_dtau"] - r64["dJ_dtau"]) <= 1e-2 * abs(r64["dJ_dtau"])
    g64, g32 = r64["dJ_dalpha"], r32["dJ_dalpha"]
    assert np.linalg.norm(g32 - g64) <= 1e-2 * np.linalg.norm(g64)


def test_autograd_function_returns_the_adjoint_gradients(cuda):
    import torch
    a = torch.tensor(alpha_field(), dtype=torch.float64, requires_grad=True)
    u = torch.tensor(U_IN, dtype=torch.float64, requires_grad=True)
    t = torch.tensor(TAU, dtype=torch.float64, requires_grad=True)
    J = drag_objective(a, u, t, case(), STEPS, K, WINDOW)
    (2.0 * J).backward()
    r = adj()
    assert float(J.detach()) == r["J"]
    assert float(u.grad) == 2.0 * r["dJ_du_in"]
    assert float(t.grad) == 2.0 * r["dJ_dtau"]
    assert np.array_equal(a.grad.numpy(), 2.0 * r["dJ_dalpha"])


def test_adjoint_rejects_bad_calls(cuda):
    with Solver(**dict(case(), storage="fp16dev", compute="fp32"), force_history=10) as s:
        with pytest.raises(cflbm.CflbmError):
            s.adjoint(10, 5, (1, 10))
    with Solver(**case(), force_history=10) as s:
        with pytest.raises(cflbm.CflbmError):
            s.adjoint(10, 5, (5, 11))   # window beyond the run
        with pytest.raises(cflbm.CflbmError):
            s.adjoint(20, 5, (1, 20))   # force history too short
        s.step(1)
        with pytest.raises(cflbm.CflbmError):
            s.adjoint(5, 5, (1, 5))     # not a fresh handle
