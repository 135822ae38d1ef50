"""GPU runs of the reference examples' own inputs against the reference's own
runs, on every column of _mc.dat.

The reference ships three Monte Carlo runs whose _mc.dat tables are the
sampled observables of its own Metropolis / parallel-tempering code:

* example01: plain Metropolis, SC 4^3 (64 sites), J1 only, 20 temperatures
  25-75 K, uniform trial moves, ferro start (examples/example01/reference/
  cubic_mc.dat);
* example02: parallel tempering, SC 14^3 (2,744 sites), 32 temperatures
  36-39.875 K around T_c, cone trial moves, swaps every 10 measurements
  (examples/example02/reference/cubic_mc.dat, swap table at
  cubic.mcout:1259-1293);
* example04: plain Metropolis, the 4-atom bmno cell 24x24x1 (2,304 sites),
  J1-J7 shells, 64 temperatures 4-70 K (examples/example04/reference/
  mc_with_uniform_temperatures/bmno_mc.dat).

Each input runs on the GPU through the library (esp_begin / esp_advance /
esp_collect, ferro start as the inputs ask), with the energy series on.
Example01 and example02 run the reference's own schedule (example02: 1e7
sweeps from the ferro start; near its first-order transition at 38.2-38.9 K
the result of a run of this length depends on the start and the length --
from a random start, or over a fifth of the schedule, the same sampler lands
up to 6 sigma away, while the reference's protocol reproduces the
reference's rows -- so the comparison keeps the protocol).  Example04's full
schedule is 2.2e12 site updates, so it runs 1/50 of it, as 4 independent
chains per temperature.  Below 8 K the plain chains relax from the ferro
start far more slowly than that schedule: after its 10^5 plain warm-up sweeps
copies still sit in different metastable states (U_M of single copies
0.37-0.42 at 4 K, their mean 0.389 against the reference's 0.373), while a
plain warm-up of 2e6 sweeps (the reference ran 5e6) gives 0.3730 +- 0.0019
and the reference's |m|, chi and E/N too (a parallel-tempering warm-up of
the short schedule does not: the slow relaxation is at the lowest
temperature itself).  So this example warms up with heat-bath moves -- the
library's learned proposal with a zero network, which for a pure exchange
Hamiltonian is the exact conditional vMF(-g/|g|, beta |g|) of every site,
accepted every time -- and then runs the reference's plain Metropolis
measurement phase from that state.  Any exact sampler of the ensemble may
warm up; the heat bath relaxes the low temperatures where a Metropolis
trial is accepted a few per cent of the time.  Per temperature the test compares
<|m|>, <E>/N, C, chi, U_E and U_M (mcarlo.F90:725-733, pt.F90:995-1024)
with the reference's row:

  z = (x_gpu - x_ref) / sqrt(sigma_gpu^2 + sigma_ref^2)

sigma_gpu is the larger of the jackknife error of the GPU's measurement
series (40 blocks, espins_gb300.analysis.jackknife_observables; combined over
the copies) and, with several copies, the spread of the copies' values (the
error of their mean), which also sees modes slower than a block -- at 4 K in
example04 the copies' spread of U_M is 8 times the jackknife error.  The
reference prints only a naive error (Delta E / Delta M, mcarlo.F90:732-733,
no autocorrelation), so its statistical error is estimated from the GPU's:
sigma_ref = sigma_gpu * sqrt(n_gpu / n_ref), n the number of measurements of
each run (the same Hamiltonian and move set, so the same error per
measurement up to the difference between typewriter and colour-class sweep
order).

The criterion is 3 sigma per comparison with a correction for the number of
comparisons K (6 observables x temperatures): every |z| <= 3, except that up
to EXCESS(K) = 1 + K * 0.0027 (rounded up; 0.27% is the two-sided 3-sigma
tail) may lie between 3 and the Bonferroni bound z_K of the family (two-sided
1% over K comparisons).  Seeds are fixed, so the outcome is deterministic;
the worst |z| per observable is printed.

Example02's replica exchange is checked twice.  From the energy series the
exact acceptance probability of every swap attempt, min(1, exp((1/T_i -
1/T_j)(E_i - E_j))) (pt.F90:1256-1283), gives each temperature's expected
acceptance; the GPU's counted acceptances must equal it within 4 sigma of the
Bernoulli noise of the decisions (a check of the exchange kernel).  That
expected acceptance, whose jackknife error over 40 blocks of attempts also
holds the slow phase dynamics near T_c, is compared with the reference's
table (pt.F90:983-990) under the same 3-sigma criterion, sigma from both
runs' jackknife errors (the reference's estimated as the GPU's, same length)
and the reference's binomial noise.
"""
import json
import math
import os

import numpy as np
import pytest

from espins_gb300 import analysis as A
from espins_gb300.lib import LP_NUM_PARAMS, Engine
from espins_gb300.tables import build_hamiltonian
from helpers import check_z, example

pytestmark = pytest.mark.gpu

SCALE = {"ex01_cubic": 1.0, "ex02_cubic_pt": 1.0, "ex04_bmno_mc": 0.02}
# examples whose warm-up is heat bath (the learned proposal with a zero network)
HEATBATH_WARMUP = {"ex04_bmno_mc"}


def copies(name, T):
    """Independent chains at temperature T."""
    return 4 if name == "ex04_bmno_mc" else 1
SEED = 20240611
BLOCKS = 40
_RUNS = {}


def _schedule(inp, scale):
    warm = max(1, int(round(inp.steps_warmup * scale)))
    mc = max(BLOCKS, int(round(inp.steps_mc * scale)))
    if inp.pt:
        pss = inp.pt_steps_swap
        mc = -(-mc // pss) * pss
        warm = -(-warm // pss) * pss
    return warm, mc


def _run(name):
    if name in _RUNS:
        return _RUNS[name]
    inp, g = example(name)
    h = build_hamiltonian(inp)
    warm, mc = _schedule(inp, SCALE[name])
    T0 = np.asarray(inp.tems, dtype=float)
    nT = T0.size
    Cs = np.array([copies(name, T) for T in T0])
    C0 = int(Cs[0])
    assert np.all(Cs == C0) and (C0 == 1 or not inp.pt)
    R = nT * C0
    # slot c * nT + t: copy c of temperature t (each copy a ladder of all temperatures)
    slot = lambda t, c: c * nT + t                  # noqa: E731
    mode = 1 if inp.mcarlo_mode.startswith("const") else 0
    with Engine(h.n, h.num_atoms, h.supercell, R, inp.boundary_open) as e:
        e.upload(h)
        e.set_temperatures(np.tile(T0, C0))
        e.init_spins("ferro")
        e.set_series(mc)
        if name in HEATBATH_WARMUP:
            # warm-up with heat-bath moves, then a new esp_begin keeps the
            # spins and starts the plain measurement phase
            e.lp_set_weights(np.zeros(LP_NUM_PARAMS, dtype=np.float32))
            e.set_proposal("learned")
            e.begin(e.schedule(warm, 1, inp.steps_measure, mode=mode, tilt=inp.tilt_angles_max, seed=SEED + 1))
            e.set_proposal("plain")
            e.begin(e.schedule(0, mc, inp.steps_measure, pt=False, mode=mode, tilt=inp.tilt_angles_max, seed=SEED))
        else:
            e.begin(e.schedule(warm, mc, inp.steps_measure, pt=inp.pt, pt_steps_swap=inp.pt_steps_swap, mode=mode,
                               tilt=inp.tilt_angles_max, seed=SEED))
        e.advance(mc // inp.pt_steps_swap if inp.pt else mc)
        res = e.collect()
        ser = e.series()
        kernel = e.sweep_kernel()[0]
    assert ser.shape == (mc, R, 2)
    n_ref = inp.steps_mc
    vals, sig, z = np.zeros((nT, 6)), np.zeros((nT, 6)), np.zeros((nT, 6))
    ref = np.array([row[1:7] for row in g["mc_dat"]])
    for t, T in enumerate(T0):
        assert abs(g["mc_dat"][t][0] - T) < 1e-3
        C = C0
        n_gpu = C * mc
        v, jk = np.zeros((C, 6)), np.zeros((C, 6))
        for c in range(C):
            k = slot(t, c)
            # the accumulators equal the moments of the series they were made from
            mom = A.moments(ser[:, k, 0], ser[:, k, 1])
            assert np.allclose(res["data"][k], mom, rtol=1e-9, atol=0.0), (T, res["data"][k], mom)
            v[c] = A.observables_of(T, res["data"][k], h.n)
            _, jk[c] = A.jackknife_observables(ser[:, k, 0], ser[:, k, 1], T, h.n, BLOCKS)
        vals[t] = v.mean(axis=0)
        sig[t] = np.sqrt((jk ** 2).sum(axis=0)) / C
        if C > 1:
            sig[t] = np.maximum(sig[t], v.std(axis=0, ddof=1) / math.sqrt(C))
        s_ref = sig[t] * math.sqrt(n_gpu / n_ref)
        z[t] = (vals[t] - ref[t]) / np.sqrt(sig[t] ** 2 + s_ref ** 2)
    out = {"name": name, "inp": inp, "g": g, "res": res, "vals": vals, "sigma": sig, "z": z, "ref": ref,
           "schedule": (warm, mc), "copies": Cs.tolist(), "kernel": kernel, "n": h.n, "series": ser}
    _RUNS[name] = out
    report = os.environ.get("ESP_STATS_REPORT")
    if report:
        os.makedirs(report, exist_ok=True)
        with open(os.path.join(report, f"reference_run_{name}.json"), "w") as fh:
            json.dump({"name": name, "schedule": [warm, mc], "copies": Cs.tolist(), "n_ref": n_ref, "kernel": kernel,
                       "tems": T0.tolist(), "observables": list(A.OBSERVABLES),
                       "gpu": vals.tolist(), "sigma_gpu": sig.tolist(), "ref": ref.tolist(), "z": z.tolist(),
                       "num_swaps": res["num_swaps"].tolist()}, fh, indent=1)
    return out


@pytest.mark.parametrize("name", list(SCALE))
def test_observables_match_the_reference_run(name):
    r = _run(name)
    z = r["z"]
    worst = {o: float(np.max(np.abs(z[:, k]))) for k, o in enumerate(A.OBSERVABLES)}
    print(f"\n{name}: schedule {r['schedule']}, copies {sorted(set(r['copies']))}, kernel {r['kernel']}, "
          f"worst |z| {worst}")
    check_z(z, lambda i: (float(r["inp"].tems[i // 6]), A.OBSERVABLES[i % 6]), name)


def _swap_expectation(ser, tems, pss, blocks=40):
    """Per temperature slot: the mean over its swap attempts of the exact
    acceptance probability, its jackknife error over `blocks` blocks of
    attempts, and the Bernoulli variance sum p(1-p) / n^2 of its decisions.
    Attempt l (1-based) follows measurement l * pss and pairs slots (0,1),
    (2,3), ... for odd l and (1,2), (3,4), ... for even l (pt.F90:898)."""
    E = ser[:, :, 0]
    R = E.shape[1]
    beta = 1.0 / np.asarray(tems, dtype=float)
    n_att = E.shape[0] // pss
    P = np.full((n_att, R), np.nan)
    for l in range(1, n_att + 1):
        e = E[l * pss - 1]
        first = 0 if l % 2 == 1 else 1
        for i in range(first, R - 1, 2):
            x = (beta[i] - beta[i + 1]) * (e[i] - e[i + 1])
            p = 1.0 if x > 0 else math.exp(x)
            P[l - 1, i] = P[l - 1, i + 1] = p
    mean = np.nanmean(P, axis=0)
    n = np.sum(~np.isnan(P), axis=0)
    bern = np.nansum(P * (1 - P), axis=0) / n ** 2
    L = n_att // blocks
    Pb = P[: blocks * L].reshape(blocks, L, R)
    bs, bc = np.nansum(Pb, axis=1), np.sum(~np.isnan(Pb), axis=1)
    loo = (bs.sum(axis=0) - bs) / (bc.sum(axis=0) - bc)
    jk = np.sqrt((blocks - 1) / blocks * ((loo - loo.mean(axis=0)) ** 2).sum(axis=0))
    return mean, jk, bern, n


def test_parallel_tempering_swap_acceptance_matches_the_reference_run():
    r = _run("ex02_cubic_pt")
    inp = r["inp"]
    sw = np.array(r["g"]["swaps"], dtype=float)
    tries, acc = r["res"]["num_swaps"][:, 0].astype(float), r["res"]["num_swaps"][:, 1].astype(float)
    # the same schedule: the reference's numbers of tries, one per temperature
    # and swap attempt it takes part in
    assert np.array_equal(tries, sw[:, 2])
    mean, jk, bern, n = _swap_expectation(r["series"], inp.tems, inp.pt_steps_swap)
    assert np.array_equal(n, tries)
    # the exchange kernel's decisions against their exact probabilities
    zk = (acc / tries - mean) / np.sqrt(bern)
    print("\nswap decisions against their probabilities, worst |z|", float(np.max(np.abs(zk))))
    assert np.all(np.abs(zk) <= 4.0), list(zip(inp.tems, acc / tries, mean, zk))
    # the expected acceptance against the reference's counted one
    theirs = sw[:, 4] / sw[:, 2]
    sig = np.sqrt(2 * jk ** 2 + theirs * (1 - theirs) / sw[:, 2])
    z = (mean - theirs) / sig
    worst = check_z(z, lambda i: (float(inp.tems[i]), "swap acceptance"), "ex02 swaps")
    print("swap acceptance against the reference, worst |z|", worst)
