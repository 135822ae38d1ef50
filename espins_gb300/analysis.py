"""Time-series analysis of Monte Carlo observables.

* ``tau_int``: integrated autocorrelation time with Sokal's automatic
  windowing (A. D. Sokal, "Monte Carlo methods in statistical mechanics:
  foundations and new algorithms", 1996): tau(M) = 1/2 + sum_{t=1..M} rho(t),
  M the smallest window with M >= c * tau(M).
* ``binning_tau``: the same quantity from the plateau of the binning analysis
  the reference runs (mcarlo.F90:548-590): tau = var_block(B) * B / (2 var(x))
  at the largest block sizes.
* ``independent_samples_per_s``: site updates/s divided by N * 2 tau_int
  (the number of sweeps between independent samples is 2 tau_int).
"""
from __future__ import annotations

import numpy as np


def autocorrelation(x: np.ndarray) -> np.ndarray:
    """Normalised autocorrelation function rho(t), t = 0..n-1, via FFT."""
    x = np.asarray(x, dtype=np.float64)
    n = x.size
    y = x - x.mean()
    f = np.fft.rfft(y, n=2 * n)
    acf = np.fft.irfft(f * np.conj(f))[:n]
    if acf[0] <= 0:
        return np.zeros(n)
    return acf / acf[0]


def tau_int(x: np.ndarray, c: float = 6.0) -> float:
    """Integrated autocorrelation time in units of the sampling interval."""
    rho = autocorrelation(x)
    tau = 0.5
    for m in range(1, rho.size):
        tau += rho[m]
        if m >= c * tau:
            return float(tau)
    return float(tau)


def binning_tau(x: np.ndarray, min_blocks: int = 32) -> float:
    """tau from the binning plateau: the largest block size with at least
    min_blocks blocks."""
    x = np.asarray(x, dtype=np.float64)
    var = x.var(ddof=1)
    if var <= 0:
        return 0.5
    best = 0.5
    b = 1
    while x.size // b >= min_blocks:
        m = x.size // b
        blocks = x[: m * b].reshape(m, b).mean(axis=1)
        best = max(best, blocks.var(ddof=1) * b / (2.0 * var))
        b *= 2
    return float(best)


def independent_samples_per_s(site_updates_per_s: float, n_sites: int, tau: float) -> float:
    """Independent samples per second of one replica's chain: sweeps/s / (2 tau)."""
    return site_updates_per_s / (n_sites * 2.0 * max(tau, 0.5))
