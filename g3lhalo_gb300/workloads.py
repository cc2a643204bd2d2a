"""Standard workloads: HOD vectors, aperture-radius triplets, binning.

HOD parameters follow the reference's device order [f, alpha, Mth, sigma, M', beta]
(src/HOD.cu:15-20).  The reference's occupation functions are
  N_c = 1/2 alpha [1 + erf(ln(m/Mth) / (sigma sqrt 2))]
  N_s = 1/2 [1 + erf(ln(m/Mth) / (sigma sqrt 2))] (m/M')^beta
(src/HOD.cu:35-76), so a model written as erf((log10 m - log10 Mth)/s) maps to
sigma = s ln10 / sqrt 2.
"""
from __future__ import annotations

import math

import numpy as np

ARCMIN_IN_RAD = 2.909e-4  # the reference's truncated constant (src/constants.h:36)
LN10 = math.log(10.0)


def hod_from_log10(log_mth: float, s_log10: float, log_m1: float, slope: float,
                   f: float = 1.0, alpha_c: float = 1.0) -> np.ndarray:
    """HOD written with log10 masses and an erf width in log10 units."""
    return np.array([f, alpha_c, 10.0 ** log_mth, s_log10 * LN10 / math.sqrt(2.0),
                     10.0 ** log_m1, slope], dtype=np.float64)


def hod_default() -> np.ndarray:
    """<Nc> = 1/2[1+erf((log m - 12)/0.2)], <Ns> = <Nc> (m/10^13.5), f = 1."""
    return hod_from_log10(12.0, 0.2, 13.5, 1.0, f=1.0)


def hod_second() -> np.ndarray:
    """Second population: log Mth 12.8, sigma 0.3, log M1 14, slope 0.9."""
    return hod_from_log10(12.8, 0.3, 14.0, 0.9, f=1.0)


def hod_sweep(n: int = 256, seed: int = 12345) -> np.ndarray:
    """n HOD vectors drawn uniformly from log Mth in [11, 13.5], sigma in [0.1, 0.6],
    log M1 in [12.5, 14.5], slope in [0.6, 1.4], f in [0.5, 1.5]."""
    rng = np.random.default_rng(seed)
    out = np.empty((n, 6))
    for i in range(n):
        lmth = rng.uniform(11.0, 13.5)
        sig = rng.uniform(0.1, 0.6)
        lm1 = rng.uniform(12.5, 14.5)
        slope = rng.uniform(0.6, 1.4)
        f = rng.uniform(0.5, 1.5)
        out[i] = hod_from_log10(lmth, sig, lm1, slope, f=f)
    return out


def theta_grid(n: int = 10, lo: float = 0.5, hi: float = 16.0) -> np.ndarray:
    """n log-spaced aperture radii in arcmin."""
    return lo * (hi / lo) ** (np.arange(n) / (n - 1))


def triplets_all(n: int = 10, lo: float = 0.5, hi: float = 16.0) -> np.ndarray:
    """All theta1 <= theta2 <= theta3 from the log grid, in radians (220 for n = 10)."""
    th = theta_grid(n, lo, hi)
    out = [(th[i], th[j], th[k]) for i in range(n) for j in range(i, n) for k in range(j, n)]
    return np.array(out, dtype=np.float64) * ARCMIN_IN_RAD


def triplets_equal(values=(0.5, 1.0, 2.0, 4.0, 8.0)) -> np.ndarray:
    """Equal-scale triplets theta1 = theta2 = theta3, in radians."""
    return np.array([(v, v, v) for v in values], dtype=np.float64) * ARCMIN_IN_RAD
