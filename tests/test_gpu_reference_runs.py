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
esp_collect, ferro start as the inputs ask), with the energy series on, for a
schedule scaled by SCALE (1 = the reference's own; example04's full schedule
is 2.2e12 site updates, so it runs 1/50 of it).  Per temperature the test
compares <|m|>, <E>/N, C, chi, U_E and U_M (mcarlo.F90:725-733,
pt.F90:995-1024) with the reference's row:

  z = (x_gpu - x_ref) / sqrt(sigma_gpu^2 + sigma_ref^2)

sigma_gpu is the jackknife error of the GPU's measurement series (40 blocks,
espins_gb300.analysis.jackknife_observables).  The reference prints only a
naive error (Delta E / Delta M, mcarlo.F90:732-733, no autocorrelation), so
its statistical error is estimated from the GPU's: sigma_ref = sigma_gpu *
sqrt(n_gpu / n_ref), n the number of measurements of each run (the same
Hamiltonian and move set, so the same error per measurement up to the
difference between typewriter and colour-class sweep order).

The criterion is 3 sigma per comparison with a correction for the number of
comparisons K (6 observables x temperatures): every |z| <= 3, except that up
to EXCESS(K) = 1 + K * 0.0027 (rounded up; 0.27% is the two-sided 3-sigma
tail) may lie between 3 and the Bonferroni bound z_K of the family (two-sided
1% over K comparisons).  Seeds are fixed, so the outcome is deterministic;
the worst |z| per observable is printed.

Example02's per-temperature swap acceptances are compared with the
reference's table under a binomial error.
"""
import json
import math
import os

import numpy as np
import pytest

from espins_gb300 import analysis as A
from espins_gb300.lib import Engine
from espins_gb300.tables import build_hamiltonian
from helpers import check_z, example

pytestmark = pytest.mark.gpu

SCALE = {"ex01_cubic": 1.0, "ex02_cubic_pt": 0.2, "ex04_bmno_mc": 0.02}
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
    R = inp.tems_num
    mode = 1 if inp.mcarlo_mode.startswith("const") else 0
    with Engine(h.n, h.num_atoms, h.supercell, R, inp.boundary_open) as e:
        e.upload(h)
        e.set_temperatures(inp.tems)
        e.init_spins("ferro")
        e.set_series(mc)
        e.begin(e.schedule(warm, mc, inp.steps_measure, pt=inp.pt, pt_steps_swap=inp.pt_steps_swap, mode=mode,
                           tilt=inp.tilt_angles_max, seed=SEED))
        e.advance(mc // inp.pt_steps_swap if inp.pt else mc)
        res = e.collect()
        ser = e.series()
        kernel = e.sweep_kernel()[0]
    assert ser.shape == (mc, R, 2)
    n_ref = inp.steps_mc
    vals, sig, z = np.zeros((R, 6)), np.zeros((R, 6)), np.zeros((R, 6))
    ref = np.array([row[1:7] for row in g["mc_dat"]])
    for t, T in enumerate(inp.tems):
        assert abs(g["mc_dat"][t][0] - T) < 1e-3
        # the accumulators equal the moments of the series they were made from
        mom = A.moments(ser[:, t, 0], ser[:, t, 1])
        assert np.allclose(res["data"][t], mom, rtol=1e-9, atol=0.0), (T, res["data"][t], mom)
        vals[t] = A.observables_of(T, res["data"][t], h.n)
        _, sig[t] = A.jackknife_observables(ser[:, t, 0], ser[:, t, 1], T, h.n, BLOCKS)
        s_ref = sig[t] * math.sqrt(mc / n_ref)
        z[t] = (vals[t] - ref[t]) / np.sqrt(sig[t] ** 2 + s_ref ** 2)
    out = {"name": name, "inp": inp, "g": g, "res": res, "vals": vals, "sigma": sig, "z": z, "ref": ref,
           "schedule": (warm, mc), "kernel": kernel, "n": h.n}
    _RUNS[name] = out
    report = os.environ.get("ESP_STATS_REPORT")
    if report:
        os.makedirs(report, exist_ok=True)
        with open(os.path.join(report, f"reference_run_{name}.json"), "w") as fh:
            json.dump({"name": name, "schedule": [warm, mc], "n_ref": n_ref, "kernel": kernel,
                       "tems": list(map(float, inp.tems)), "observables": list(A.OBSERVABLES),
                       "gpu": vals.tolist(), "sigma_gpu": sig.tolist(), "ref": ref.tolist(), "z": z.tolist(),
                       "num_swaps": res["num_swaps"].tolist()}, fh, indent=1)
    return out


@pytest.mark.parametrize("name", list(SCALE))
def test_observables_match_the_reference_run(name):
    r = _run(name)
    z = r["z"]
    worst = {o: float(np.max(np.abs(z[:, k]))) for k, o in enumerate(A.OBSERVABLES)}
    print(f"\n{name}: schedule {r['schedule']} kernel {r['kernel']} worst |z| {worst}")
    check_z(z, lambda i: (float(r["inp"].tems[i // 6]), A.OBSERVABLES[i % 6]), name)


def test_parallel_tempering_swap_acceptance_matches_the_reference_run():
    """Per temperature: accepted / tried swaps against the reference's
    example02 table (pt.F90:983-990), binomial sigma of both runs, 4 sigma
    (32 comparisons)."""
    r = _run("ex02_cubic_pt")
    sw = np.array(r["g"]["swaps"], dtype=float)
    tries, acc = r["res"]["num_swaps"][:, 0].astype(float), r["res"]["num_swaps"][:, 1].astype(float)
    assert np.all(tries > 0)
    ours = acc / tries
    theirs = sw[:, 4] / sw[:, 2]
    p = np.clip(0.5 * (ours + theirs), 1e-3, 1 - 1e-3)
    # consecutive swap decisions are correlated through the energies; a factor
    # 2 on the binomial error covers their autocorrelation
    sig = 2.0 * np.sqrt(p * (1 - p) * (1.0 / tries + 1.0 / sw[:, 2]))
    zz = (ours - theirs) / sig
    print("\nswap acceptance worst |z|", float(np.max(np.abs(zz))))
    assert np.all(np.abs(zz) <= 4.0), list(zip(r["inp"].tems, ours, theirs, zz))
    # the reference counts one try per temperature and swap attempt it takes part in
    inner = tries[1:-1]
    assert np.all(inner == inner[0]) and tries[0] == tries[-1]
