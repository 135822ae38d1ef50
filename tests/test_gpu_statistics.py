"""Statistical parity: GPU colour-class chains against the oracle's typewriter
chains (the reference's algorithm: mcarlo.F90:496-733, pt.F90:504-1024).

The two samplers use different site orders and random streams, so only
stationary averages can agree.  For every temperature the test averages
independent chains (COPIES replicas on the GPU, ORACLE_CHAINS typewriter
chains on the CPU) and requires |<x>_gpu - <x>_oracle| <= 3 sigma for
x = E/N and |m|, with sigma combined from every chain's binning analysis
(mcarlo.F90:635-656): the largest of the binning error estimates over block
sizes 2^5..2^9.  The derived columns of _mc.dat -- C, chi and the Binder
cumulants U_E, U_M (mcarlo.F90:725-731) -- are compared the same way, with
the GPU chains' jackknife errors (40 blocks of each chain's measurement
series) and, for the oracle's chains, whose series are not kept, the GPU
chains' error per chain (same chain length and move set) scaled to the
number of oracle chains.  Over all temperatures and observables of a test the
3-sigma criterion of helpers.check_z applies.  Seeds are fixed, so the
outcome is deterministic.
"""
import numpy as np
import pytest

import oracle as O
from espins_gb300 import analysis as A
from espins_gb300.lib import Engine
from espins_gb300.tables import build_hamiltonian
from helpers import NN, NNN, check_z, energy_scale, sc_mcin

pytestmark = pytest.mark.gpu

LEVELS = [1, 2, 3, 4, 5, 6, 7, 8, 9]
COPIES = 4
ORACLE_CHAINS = 2


def _sigma(binning):
    """binning: (levels, 2) variances of the mean of E/N and |m|."""
    b = np.asarray(binning)[4:9]
    return np.sqrt(np.max(np.maximum(b, 0.0), axis=0))


def _gpu_run(h, tems, pt, warm, mc, pss=10, mode=0, tilt=0.125, seed=12345):
    R = len(tems)
    with Engine(h.n, h.num_atoms, h.supercell, R) as e:
        e.upload(h)
        e.set_temperatures(tems)
        e.init_spins("ferro")
        e.set_series(mc)
        res = e.run(warm, mc, 1, pt=pt, pt_steps_swap=pss, mode=mode, tilt=tilt, seed=seed,
                    binning_level=LEVELS)
        res["series"] = e.series()
    assert res["series"].shape[0] == mc
    return res


DERIVED = ("C", "chi", "U_E", "U_M")


def _derived(T, n, gpu_series, or_data):
    """C, chi, U_E, U_M: (mean over GPU chains, its sigma) and (mean over the
    oracle's chains, its estimated sigma).  gpu_series: list of (E, |m|)
    series per GPU chain; or_data: list of normalised accumulators (6,)."""
    gv, gs = [], []
    for ser in gpu_series:
        v, s = A.jackknife_observables(ser[:, 0], ser[:, 1], T, n, 40)
        gv.append(v[2:]); gs.append(s[2:])
    gv, gs = np.array(gv), np.array(gs)
    ov = np.array([A.observables_of(T, d, n)[2:] for d in or_data])
    per_chain = np.sqrt((gs ** 2).mean(axis=0))
    return gv.mean(axis=0), np.sqrt((gs ** 2).sum(axis=0)) / len(gv), ov.mean(axis=0), per_chain / np.sqrt(len(ov))


def _check_derived(h, tems, gpu_series, or_data, what):
    """gpu_series[t]: per-chain (E, |m|) series; or_data[t]: per-chain accumulators."""
    z = np.zeros((len(tems), len(DERIVED)))
    for t, T in enumerate(tems):
        g, sg, o, so = _derived(T, h.n, gpu_series[t], or_data[t])
        z[t] = (g - o) / np.sqrt(sg ** 2 + so ** 2)
    worst = check_z(z, lambda i: (float(tems[i // len(DERIVED)]), DERIVED[i % len(DERIVED)]), what)
    print(f"\n{what}: worst |z| of C, chi, U_E, U_M = {worst:.2f}")


def _mean_sigma(datas, bins, n):
    """Mean of independent chains' <E/N>, <|m|> and the sigma of that mean."""
    x = np.array([[d[0] / n, d[3]] for d in datas])
    s = np.array([_sigma(b) for b in bins])
    return x.mean(axis=0), np.sqrt((s ** 2).sum(axis=0)) / len(datas)


def _check(h, tems, gpu_data, gpu_bin, or_data, or_bin, what):
    """gpu_*/or_*: per temperature, lists of per-chain data (6,) and binning (levels, 2)."""
    n = h.n
    for t, T in enumerate(tems):
        g, sg = _mean_sigma(gpu_data[t], gpu_bin[t], n)
        o, so = _mean_sigma(or_data[t], or_bin[t], n)
        s = np.sqrt(sg ** 2 + so ** 2)
        assert np.all(np.abs(g - o) <= 3.0 * s), (what, T, g, o, s)


def _gpu_copies(h, tems, warm, mc, **kw):
    """COPIES independent replicas per temperature in one GPU run (plain)."""
    rt = np.repeat(np.asarray(tems, dtype=float), COPIES)
    res = _gpu_run(h, rt, False, warm, mc, **kw)
    d = res["data"].reshape(len(tems), COPIES, 6)
    b = res["binning"].reshape(len(tems), COPIES, len(LEVELS), 2)
    e = res["energy"]
    ser = res["series"].reshape(mc, len(tems), COPIES, 2)
    series = [[ser[:, t, c, :] for c in range(COPIES)] for t in range(len(tems))]
    return [list(x) for x in d], [list(x) for x in b], e, series


def _oracle_chains(h, tems, warm, mc, seed0, **kw):
    H = O.Ham(h)
    datas, bins = [], []
    for t, T in enumerate(tems):
        dd, bb = [], []
        for c in range(ORACLE_CHAINS):
            s = np.zeros((h.n, 3)); s[:, 2] = 1.0
            r = H.mcarlo(O.MT(seed0 + 100 * c + t), 1.0 / T, s, warm, mc, 1, binning_level=LEVELS,
                         want_pm=False, **kw)
            dd.append(r["data"] / mc)
            bb.append(r["binning"])
        datas.append(dd); bins.append(bb)
    return datas, bins


@pytest.mark.parametrize("mode", [0, 1])
def test_plain_metropolis_matches_reference_algorithm(mode):
    inp = sc_mcin(6, [(1e-3, NN)], [8.0, 14.0, 20.0, 30.0])
    h = build_hamiltonian(inp)
    tems = inp.tems
    warm, mc = 2000, 40000
    gd, gb, e, gs = _gpu_copies(h, tems, warm, mc, mode=mode, tilt=0.3)
    od, ob = _oracle_chains(h, tems, warm, mc, 1000, mode=mode, tilt=0.3)
    _check(h, tems, gd, gb, od, ob, f"plain mode={mode}")
    _check_derived(h, tems, gs, od, f"plain mode={mode}")
    # the energy bookkeeping of the run: final by differences == direct, up to
    # the FP32 rounding of ~1e7 accumulated energy differences
    assert np.max(np.abs(e[:, 1] - e[:, 2])) <= 1e-5 * energy_scale(h)


def test_plain_metropolis_biquadratic_dm_singleion():
    inp = sc_mcin(6, [(1e-3, NN), (3e-4, NNN)], [5.0, 12.0, 25.0], bq=1e-4, dm=2e-4, si=-3e-5)
    h = build_hamiltonian(inp)
    tems = inp.tems
    warm, mc = 2000, 30000
    gd, gb, _, gs = _gpu_copies(h, tems, warm, mc)
    od, ob = _oracle_chains(h, tems, warm, mc, 77)
    _check(h, tems, gd, gb, od, ob, "J+B+D+SI")
    _check_derived(h, tems, gs, od, "J+B+D+SI")


def test_parallel_tempering_matches_reference_algorithm():
    inp = sc_mcin(6, [(1e-3, NN)], list(np.geomspace(8.0, 30.0, 8)))
    h = build_hamiltonian(inp)
    tems = inp.tems
    warm, mc, pss = 4000, 40000, 10
    res = _gpu_run(h, tems, True, warm, mc, pss=pss)
    H = O.Ham(h)
    s = np.zeros((len(tems), h.n, 3)); s[:, :, 2] = 1.0
    r = H.pt(O.MT(4242), tems, s.reshape(-1), warm, mc, 1, pss, binning_level=LEVELS, want_pm=False)
    steps = r["steps_mc_eff"]
    or_data = r["data"] / steps
    # PT binning variances carry an extra 1/N (pt.F90:935); undo it for sigma
    gb = res["binning"] * h.n
    ob = r["binning"] * h.n
    _check(h, tems, [[d] for d in res["data"]], [[b] for b in gb], [[d] for d in or_data], [[b] for b in ob], "pt")
    _check_derived(h, tems, [[res["series"][:, t, :]] for t in range(len(tems))], [[d] for d in or_data], "pt")
    # swap acceptance per temperature: binomial tolerance
    ga = res["num_swaps"][:, 1] / np.maximum(res["num_swaps"][:, 0], 1)
    oa = r["num_swaps"][:, 1] / np.maximum(r["num_swaps"][:, 0], 1)
    ntries = np.maximum(res["num_swaps"][:, 0], 1)
    sig = np.sqrt(np.maximum(oa * (1 - oa), 1e-4) / ntries) * 2.0
    assert np.all(np.abs(ga - oa) <= 4 * sig + 0.02), (ga, oa)
    # map is a permutation, tries are counted as the reference counts them
    assert sorted(res["map"].tolist()) == list(range(1, len(tems) + 1))
    nsw = steps // pss
    assert res["num_swaps"][0, 0] == (nsw + 1) // 2
