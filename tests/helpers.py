"""Shared helpers of the tests: fixtures of the reference examples and small
synthetic lattices with the shapes of the benchmark configurations."""
import json
import os

import numpy as np

from espins_gb300.mcin import K_B, parse_mcin, read_mcin
from espins_gb300.tables import build_hamiltonian

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def example(name, nodes=None):
    if nodes is None:
        nodes = 32 if name.startswith(("ex02", "ex04")) else 4
    inp = read_mcin(os.path.join(GOLDEN, name + ".mcin"), num_nodes=nodes)
    with open(os.path.join(GOLDEN, name + "_golden.json")) as fh:
        g = json.load(fh)
    return inp, g


def example_spins(name):
    z = np.load(os.path.join(GOLDEN, name + "_sconfig.npz"))
    return z["temps"], z["spins"]


def sc_mcin(L, shells, tems, extra="", bq=None, dm=None, si=None, steps=(100, 1000, 1)):
    """A simple-cubic input: shells = [(J_eV, offsets...)], optional NN biquadratic
    (eV), NN DM (eV, along the unit bond vector) and single-ion (Delta eV along z)."""
    lines = ["begin unit_cell_cart", "1 0 0", "0 1 0", "0 0 1", "end unit_cell_cart",
             "begin atoms_frac", "Fe 0 0 0 1.0", "end atoms_frac",
             f"supercell_size = {L} {L} {L}", "tems_mode = man", f"tems_num = {len(tems)}",
             "tems = " + " ".join(repr(float(t)) for t in tems),
             f"steps_warmup = {steps[0]}", f"steps_mc = {steps[1]}", f"steps_measure = {steps[2]}"]
    lines.append("begin jij_parameters")
    for J, offs in shells:
        for o in offs:
            lines.append(f"f1=0,0,0:f2={o[0]},{o[1]},{o[2]}:jij={J}")
    lines.append("end jij_parameters")
    nn = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]
    if bq is not None:
        lines += ["ham_bij = .true.", "begin bij_parameters"]
        lines += [f"f1=0,0,0:f2={o[0]},{o[1]},{o[2]}:bij={bq}" for o in nn]
        lines.append("end bij_parameters")
    if dm is not None:
        lines += ["ham_dij = .true.", "begin dij_parameters"]
        lines += [f"f1=0,0,0:f2={o[0]},{o[1]},{o[2]}:dij={dm}" for o in nn]
        lines += ["end dij_parameters", "begin dij_vectors_cart"]
        lines += [f"{o[0]} {o[1]} {o[2]}" for o in nn]
        lines.append("end dij_vectors_cart")
    if si is not None:
        lines += ["ham_singleion = .true.", "begin singleion_axes_cart", f"Fe 0 0 1 {si}", "end singleion_axes_cart"]
    lines += [l for l in extra.splitlines() if l.strip()]
    return parse_mcin("\n".join(lines) + "\n", seedname="sc")


NN = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]
NNN = [(a, b, 0) for a in (1, -1) for b in (1, -1)] + [(a, 0, b) for a in (1, -1) for b in (1, -1)] + \
      [(0, a, b) for a in (1, -1) for b in (1, -1)]
N3 = [(a, b, c) for a in (1, -1) for b in (1, -1) for c in (1, -1)]


# FP32 site arithmetic against the FP64 oracle: errors relative to the
# coupling-magnitude scales below (energy_scale for totals, site_scale per
# site).  Measured on GB300 over the reference examples and the benchmark
# Hamiltonians: at most 4.1e-8 for totals and 3.9e-7 for local fields.
ENERGY_RTOL = 1e-6
FIELD_RTOL = 1e-6


def energy_scale(h):
    """Sum of |coupling| magnitudes: the floor for relative energy errors."""
    s = 0.5 * np.abs(h.jij.val).sum()
    if h.bij is not None:
        s += 0.5 * np.abs(h.bij.val).sum()
    if h.dij is not None:
        s += 0.5 * np.abs(h.dij.val).sum()
    if h.si_delta is not None:
        s += h.n * np.abs(h.si_delta).max()
    return s


def site_scale(h):
    """Per-site sum of |J| + |B| + |D| (floor for local-field errors)."""
    sc = np.abs(h.jij.val).sum(axis=0)
    if h.bij is not None:
        sc = sc + np.abs(h.bij.val).sum(axis=0)
    if h.dij is not None:
        sc = sc + np.abs(h.dij.val).sum(axis=(0, 2))
    if h.si_delta is not None:
        sc = sc + np.abs(h.si_delta).max()
    return sc


def bonferroni_z(K, alpha=0.01):
    """Two-sided normal bound z with K * P(|Z| > z) = alpha."""
    import math
    lo, hi = 0.0, 10.0
    for _ in range(100):
        mid = 0.5 * (lo + hi)
        if K * math.erfc(mid / math.sqrt(2.0)) > alpha:
            lo = mid
        else:
            hi = mid
    return hi


def check_z(z, labels, what):
    """The 3-sigma criterion of the statistical tests over K = z.size
    comparisons: every |z| <= 3, except that up to ceil(1 + 0.0027 K) of them
    (0.27% is the two-sided 3-sigma tail) may lie between 3 and the Bonferroni
    bound of the family (two-sided 1% over K).  labels(i) names comparison i
    of the flattened z.  Returns the worst |z|."""
    import math
    az = np.abs(np.asarray(z, dtype=float)).reshape(-1)
    assert np.all(np.isfinite(az)), (what, z)
    K = az.size
    over = [(labels(i), float(az[i])) for i in np.nonzero(az > 3.0)[0]]
    assert len(over) <= math.ceil(1 + 0.0027 * K), (what, over)
    zK = bonferroni_z(K)
    assert np.all(az <= zK), (what, zK, over)
    return float(az.max()) if K else 0.0


def exact_energy_axial(F, D, T, n=2_000_000):
    """<E> per site of E(s) = F s_z + D s_x^2 on the unit sphere: the azimuth
    integral of exp(-D sin^2(t) cos^2(p) / T) is 2 pi exp(-a) I0(a) with
    a = D sin^2(t) / (2T), leaving a fine one-dimensional integral over
    cos(t)."""
    from scipy.special import i0e
    u = -1 + (np.arange(n) + 0.5) * (2.0 / n)
    s2 = 1 - u * u
    a = D * s2 / (2 * T)
    # weight exp(-F u / T) * exp(-a) I0(a) and <s_x^2> = sin^2 * <cos^2 p>
    # with <cos^2 p> = (1 - I1(a)/I0(a)) / 2 under exp(-2a cos^2 p)
    from scipy.special import i1e
    lw = -(F * u) / T + np.log(i0e(a))
    w = np.exp(lw - lw.max())
    cos2 = 0.5 * (1 - i1e(a) / i0e(a))
    e = F * u + D * s2 * cos2
    return float((e * w).sum() / w.sum())
