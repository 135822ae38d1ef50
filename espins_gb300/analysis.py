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


# Columns of _mc.dat after the temperature (mcarlo.F90:725-733, pt.F90:995-1024):
# <|m|>, <E>/N, C, chi, U_E, U_M
OBSERVABLES = ("absM", "E_per_site", "C", "chi", "U_E", "U_M")


def moments(E: np.ndarray, absm: np.ndarray) -> np.ndarray:
    """The six accumulators of one measurement series, normalised as the
    reference normalises them: <E>, <E^2>, <E^4>, <|m|>, <m^2>, <m^4>."""
    E = np.asarray(E, dtype=np.float64)
    m = np.asarray(absm, dtype=np.float64)
    E2, m2 = E * E, m * m
    return np.array([E.mean(), E2.mean(), (E2 * E2).mean(), m.mean(), m2.mean(), (m2 * m2).mean()])


def observables_of(T: float, row: np.ndarray, n: int) -> np.ndarray:
    """<|m|>, <E>/N, C, chi, U_E, U_M from the normalised accumulators."""
    beta = 1.0 / T
    E, E2, E4, M, M2, M4 = row
    return np.array([M, E / n, beta * beta * (E2 - E * E) / n, beta * (M2 - M * M) * n,
                     1.0 - E4 / (3.0 * E2 * E2), 1.0 - M4 / (3.0 * M2 * M2)])


def jackknife_observables(E: np.ndarray, absm: np.ndarray, T: float, n: int, blocks: int = 40):
    """Values and jackknife errors of the _mc.dat observables from one series
    of (E, |m|) per measurement: the series is cut into `blocks` consecutive
    blocks (each much longer than the autocorrelation time, so blocks are
    nearly independent); each block is left out in turn and the observables
    recomputed from the remaining measurements' moments;
    sigma^2 = (B - 1) / B * sum_b (theta_b - mean theta)^2.  The values are
    those of the whole series.  Returns (values (6,), sigma (6,))."""
    E = np.asarray(E, dtype=np.float64)
    m = np.asarray(absm, dtype=np.float64)
    B = int(blocks)
    L = E.size // B
    if L < 1:
        raise ValueError("series shorter than the number of blocks")
    E, m = E[: B * L], m[: B * L]
    E2, m2 = E * E, m * m
    cols = np.stack([E, E2, E2 * E2, m, m2, m2 * m2], axis=1)       # (B*L, 6)
    bsum = cols.reshape(B, L, 6).sum(axis=1)                        # (B, 6)
    tot = bsum.sum(axis=0)
    full = observables_of(T, tot / (B * L), n)
    loo = np.array([observables_of(T, (tot - bsum[b]) / ((B - 1) * L), n) for b in range(B)])
    sigma = np.sqrt((B - 1) / B * ((loo - loo.mean(axis=0)) ** 2).sum(axis=0))
    return full, sigma
