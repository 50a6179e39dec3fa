"""Gradients of the time-averaged drag (or lift) of a D2Q9 channel.

`drag_objective` is a torch.autograd.Function: its forward runs the solver and
the hand-written adjoint sweep (cflbm_adjoint in libcflbm.so) once, returns J,
and its backward hands back dJ/dalpha, dJ/du_in and dJ/dtau scaled by the
incoming gradient.  torch is only the front end here: nothing is computed by it.
"""
from __future__ import annotations

import numpy as np

from .solver import Solver


def smooth_porosity(nx: int, ny: int, box: tuple[int, int, int, int], seed: int,
                    n_bumps: int = 8, widths: tuple[float, float] = (8.0, 24.0)) -> np.ndarray:
    """Seeded smooth porosity field in [0, 1]: the sum of `n_bumps` Gaussians with
    widths drawn from `widths`, centred inside `box` = (x0, y0, x1, y1) (half-open),
    scaled so its maximum is 1, and zero outside the box."""
    rng = np.random.default_rng(seed)
    x0, y0, x1, y1 = box
    X, Y = np.meshgrid(np.arange(x0, x1), np.arange(y0, y1))
    acc = np.zeros(X.shape)
    for _ in range(n_bumps):
        cx, cy = rng.uniform(x0, x1), rng.uniform(y0, y1)
        s = rng.uniform(*widths)
        amp = rng.uniform(0.5, 1.0)
        acc += amp * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2.0 * s * s))
    acc /= acc.max()
    out = np.zeros((ny, nx))
    out[y0:y1, x0:x1] = acc
    return out


def run(case: dict, alpha: np.ndarray | None, u_in: float, tau: float, steps: int,
        checkpoint_every: int, window: tuple[int, int], objective: str = "drag") -> dict:
    """One forward + adjoint run.  `case` holds the other Solver keywords (grid,
    geometry, walls, storage/compute, perturbation); tau is the relaxation time
    tau0 + 0.5."""
    kw = dict(case)
    kw.update(u0=float(u_in), tau0=float(tau) - 0.5, force_history=int(steps))
    if alpha is not None:
        kw["alpha"] = np.asarray(alpha, dtype=np.float64)
    with Solver(**kw) as s:
        return s.adjoint(steps, checkpoint_every, window, objective)


def _function():
    import torch

    class DragObjective(torch.autograd.Function):
        """J(alpha, u_in, tau) = mean force over the window; backward = the adjoint."""

        @staticmethod
        def forward(ctx, alpha, u_in, tau, case, steps, checkpoint_every, window, objective):
            r = run(case, alpha.detach().cpu().double().numpy(), float(u_in), float(tau),
                    steps, checkpoint_every, window, objective)
            ctx.save_for_backward(
                torch.as_tensor(r["dJ_dalpha"], dtype=alpha.dtype, device=alpha.device),
                torch.tensor(r["dJ_du_in"], dtype=u_in.dtype, device=u_in.device),
                torch.tensor(r["dJ_dtau"], dtype=tau.dtype, device=tau.device))
            ctx.result = r
            return torch.tensor(r["J"], dtype=torch.float64, device=alpha.device)

        @staticmethod
        def backward(ctx, gJ):
            ga, gu, gt = ctx.saved_tensors
            return (gJ.to(ga.dtype) * ga, gJ.to(gu.dtype) * gu, gJ.to(gt.dtype) * gt,
                    None, None, None, None, None)

    return DragObjective


_FN = None


def drag_objective(alpha, u_in, tau, case: dict, steps: int, checkpoint_every: int = 100,
                   window: tuple[int, int] | None = None, objective: str = "drag"):
    """torch front end: alpha (ny, nx), u_in and tau (0-d) tensors -> J (0-d).
    J.backward() fills their .grad from one adjoint sweep."""
    global _FN
    if _FN is None:
        _FN = _function()
    if window is None:
        window = (1, steps)
    return _FN.apply(alpha, u_in, tau, case, steps, checkpoint_every, tuple(window), objective)
