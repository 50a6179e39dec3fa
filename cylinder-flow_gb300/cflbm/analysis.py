"""Post-processing of the force history: Cd/Cl statistics and the Strouhal number.

The reference writes the per-step "Cd Cl" pair to test.dat
("MPI Kokkos/lbm.cpp:398-407") and computes no Strouhal number; this module
adds St = f_shed D / u0 from the lift series, and writes test.dat lines in the
reference's format (fixed, 17 digits).
"""
from __future__ import annotations

import numpy as np


def coefficients(force: np.ndarray, u0: float, area: float) -> np.ndarray:
    """(steps, 2) array of (Cd, Cl) = 2 F / (u0^2 A) from (steps, >=2) forces."""
    f = np.asarray(force, np.float64)
    return 2.0 * f[:, :2] / (u0 * u0 * area)


def strouhal(cl: np.ndarray, diam: float, u0: float, dt: float = 1.0) -> float:
    """Shedding Strouhal number from a lift-coefficient series.

    The dominant frequency is the peak of the periodogram of the detrended,
    Hann-windowed series, refined by a parabola through the peak bin and its two
    neighbours (in log power).  Returns nan when no oscillation is present.
    """
    x = np.asarray(cl, np.float64)
    n = x.size
    if n < 16 or not np.all(np.isfinite(x)):
        return float("nan")
    t = np.arange(n)
    x = x - np.polyval(np.polyfit(t, x, 1), t)
    if np.max(np.abs(x)) < 1e-14:
        return float("nan")
    w = np.hanning(n)
    spec = np.abs(np.fft.rfft(x * w)) ** 2
    spec[0] = 0.0
    k = int(np.argmax(spec))
    if k <= 0 or k >= spec.size - 1:
        return float("nan")
    a, b, c = np.log(spec[k - 1] + 1e-300), np.log(spec[k] + 1e-300), np.log(spec[k + 1] + 1e-300)
    denom = a - 2 * b + c
    delta = 0.5 * (a - c) / denom if denom != 0 else 0.0
    freq = (k + delta) / (n * dt)
    return float(freq * diam / u0)


def shedding_window(cl: np.ndarray, diam: float, u0: float) -> tuple[int, int]:
    """(start, periods): the last whole shedding periods of a lift series -- the
    period from the Strouhal number (the periodogram peak, robust to noise on
    the lift), the largest whole number of periods that fits, counted back from
    the series' end.  (0, 0) when the lift does not oscillate."""
    st = strouhal(cl, diam, u0)
    n = np.asarray(cl).size
    if not np.isfinite(st) or st <= 0.0:
        return 0, 0
    period = diam / (st * u0)  # steps
    k = int(n // period)
    if k < 1:
        return 0, 0
    return n - int(round(k * period)), k


def summary(force: np.ndarray, u0: float, area: float, diam: float, window: int | None = None):
    """Mean Cd, rms Cl and St over the last `window` steps.

    cd_mean is the plain window mean.  cd_mean_periods averages the drag over
    the last whole shedding periods inside the window (shedding_window): in
    periodic shedding the drag oscillates at twice the shedding frequency, and a
    window that ends mid-cycle moves the plain mean by a part of that
    oscillation's amplitude -- so two runs whose shedding phases differ by a
    fraction of a period differ in cd_mean without differing in mean drag.
    Equal to cd_mean when the lift does not oscillate."""
    cc = coefficients(force, u0, area)
    if window:
        cc = cc[-window:]
    cd, cl = cc[:, 0], cc[:, 1]
    a, n = shedding_window(cl, diam, u0)
    return {
        "cd_mean": float(np.mean(cd)),
        "cd_mean_periods": float(np.mean(cd[a:])) if n else float(np.mean(cd)),
        "periods": n,
        "cl_rms": float(np.sqrt(np.mean((cl - np.mean(cl)) ** 2))),
        "st": strouhal(cl, diam, u0),
        "steps": int(cc.shape[0]),
    }


def write_test_dat(path: str, cd_cl: np.ndarray, append: bool = True) -> None:
    """Append "Cd Cl" lines exactly as the reference's test.dat (fixed, 17 digits)."""
    with open(path, "a" if append else "w") as fh:
        for cd, cl in np.asarray(cd_cl, np.float64).reshape(-1, 2):
            fh.write(f"{cd:.17f} {cl:.17f}\n")
