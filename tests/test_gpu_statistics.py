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
from helpers import NN, NNN, check_z, energy_scale, exact_energy_axial, sc_mcin

pytestmark = pytest.mark.gpu

LEVELS = [1, 2, 3, 4, 5, 6, 7, 8, 9]
COPIES = 4
ORACLE_CHAINS = 2
PT_CHAINS = 4


def _sigma(binning):
    """binning: (levels, 2) variances of the mean of E/N and |m|."""
    b = np.asarray(binning)[4:9]
    return np.sqrt(np.max(np.maximum(b, 0.0), axis=0))


def _gpu_run(h, tems, pt, warm, mc, pss=10, mode=0, tilt=0.125, seed=12345, pt_group=None):
    R = len(tems)
    with Engine(h.n, h.num_atoms, h.supercell, R) as e:
        e.upload(h)
        e.set_temperatures(tems)
        if pt_group:
            e.set_pt_groups(pt_group)
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


@pytest.mark.parametrize("mode", [0, 1])
def test_plain_sampler_is_exact_on_independent_sites(mode):
    """The plain Metropolis move (uniform or cone trial spin, Boltzmann test:
    metropolis, get_quant.F90:52-182) on sites without couplings in a 100 T
    field along z (67 K) with an easy-plane term along x, at 0.5-8 K:
    <E>/N of COPIES replicas per temperature against a fine quadrature of
    the exact single-site distribution.  An answer with no run in between,
    sharp enough (sigma ~1e-3 K) to see a bias of the trial direction or of
    the acceptance test."""
    tems = [0.5, 2.0, 8.0]
    extra = ("ham_field = .true.\nbegin field_axes_cart\nFe 0 0 1 100.0\nend field_axes_cart\n"
             "ham_singleion = .true.\nbegin singleion_axes_cart\nFe 1 0 0 2e-4\nend singleion_axes_cart\n")
    inp = sc_mcin(6, [(1e-12, NN)], tems, extra=extra)
    h = build_hamiltonian(inp)
    F = float(h.field_val[0] * h.field_axis[0][2])
    D = float(h.si_delta[0])
    gd, gb, _, _ = _gpu_copies(h, tems, 2000, 20000, mode=mode, tilt=0.3)
    for t, T in enumerate(tems):
        g, sg = _mean_sigma(gd[t], gb[t], h.n)
        want = exact_energy_axial(F, D, T)
        print(f"\nmode {mode} T={T}: E/N {g[0]:.6f} +- {sg[0]:.6f}, exact {want:.6f}")
        assert abs(g[0] - want) <= 3 * sg[0] + 1e-6 * abs(want), (mode, T, g[0], want, sg[0])


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
    """PT_CHAINS independent parallel-tempering chains on the GPU (replica
    groups of one handle) against the oracle's chain.  The error of the GPU's
    mean is the larger of the chains' combined binning error and their
    spread; the oracle's chain, as long as each GPU chain and of the same
    algorithm, is given at least a GPU chain's error (the spread times
    sqrt(PT_CHAINS)), since its binning blocks (at most 2^9 measurements) can
    be shorter than the exchange's slowest mode at the lowest temperature."""
    inp = sc_mcin(6, [(1e-3, NN)], list(np.geomspace(8.0, 30.0, 8)))
    h = build_hamiltonian(inp)
    tems = np.asarray(inp.tems)
    nT = len(tems)
    warm, mc, pss = 4000, 40000, 10
    res = _gpu_run(h, np.tile(tems, PT_CHAINS), True, warm, mc, pss=pss, pt_group=nT)
    H = O.Ham(h)
    s = np.zeros((nT, h.n, 3)); s[:, :, 2] = 1.0
    r = H.pt(O.MT(4242), tems, s.reshape(-1), warm, mc, 1, pss, binning_level=LEVELS, want_pm=False)
    steps = r["steps_mc_eff"]
    or_data = r["data"] / steps
    # PT binning variances carry an extra 1/N (pt.F90:935); undo it for sigma
    gb = (res["binning"] * h.n).reshape(PT_CHAINS, nT, len(LEVELS), 2)
    ob = r["binning"] * h.n
    gd = res["data"].reshape(PT_CHAINS, nT, 6)
    for t, T in enumerate(tems):
        x = np.array([[gd[c, t, 0] / h.n, gd[c, t, 3]] for c in range(PT_CHAINS)])
        sb = np.array([_sigma(gb[c, t]) for c in range(PT_CHAINS)])
        spread = x.std(axis=0, ddof=1)
        sg = np.maximum(np.sqrt((sb ** 2).sum(axis=0)) / PT_CHAINS, spread / np.sqrt(PT_CHAINS))
        o = np.array([or_data[t, 0] / h.n, or_data[t, 3]])
        so = np.maximum(_sigma(ob[t]), np.maximum(np.sqrt((sb ** 2).mean(axis=0)), spread))
        z = (x.mean(axis=0) - o) / np.sqrt(sg ** 2 + so ** 2)
        assert np.all(np.abs(z) <= 3.0), ("pt", T, x.mean(axis=0), o, sg, so)
    ser = res["series"].reshape(-1, PT_CHAINS, nT, 2)
    _check_derived(h, tems, [[ser[:, c, t, :] for c in range(PT_CHAINS)] for t in range(nT)],
                   [[d] for d in or_data], "pt")
    # swap acceptance per temperature (first chain): binomial tolerance
    ns = res["num_swaps"][:nT]
    ga = ns[:, 1] / np.maximum(ns[:, 0], 1)
    oa = r["num_swaps"][:, 1] / np.maximum(r["num_swaps"][:, 0], 1)
    ntries = np.maximum(ns[:, 0], 1)
    sig = np.sqrt(np.maximum(oa * (1 - oa), 1e-4) / ntries) * 2.0
    assert np.all(np.abs(ga - oa) <= 4 * sig + 0.02), (ga, oa)
    # map is a permutation within each chain, tries are counted as the reference counts them
    for c in range(PT_CHAINS):
        assert sorted(res["map"][c * nT:(c + 1) * nT].tolist()) == list(range(c * nT + 1, (c + 1) * nT + 1))
    nsw = steps // pss
    assert ns[0, 0] == (nsw + 1) // 2
