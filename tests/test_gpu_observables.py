"""The order parameter, the staggered magnetisation and the spin correlations
measured on the GPU (orderparam_get, staggered_get, Pm_get's pdf_order /
pdf_staggered and spincorr_get, get_quant.F90:366-540, accumulated as
mcarlo.F90:545-590 / pt.F90:798-849):

* every sweep kernel's measurements equal the oracle's evaluation of the same
  spins, measurement by measurement (accumulators, binning, P(OP), P(SM));
* the cluster-resident kernel (in-kernel measurement) and the ELL path agree
  on a parallel-tempering run;
* staggered coefficients of +1 reproduce the magnetisation columns;
* the stationary averages of <|OP|> and <SM> agree with the oracle's
  typewriter chains (the reference's algorithm) within 3 sigma;
* the spin correlations equal the oracle's spincorr_get of the same spins,
  measurement by measurement, for every sweep kernel;
* the structure factor equals the oracle's mcarlo_structure_factor of the
  same spins on every measurement that is a multiple of its cadence;
* the host driver writes _op.dat, _staggered.dat, _spincorr.dat, the extra
  columns and the energy series files (whose rows do not depend on how the
  run is chunked, and whose last row is the final running energy).
"""
import os

import numpy as np
import pytest

import oracle as O
from espins_gb300 import mc
from espins_gb300.lib import Engine
from espins_gb300.tables import build_hamiltonian, build_shells, sfactor_qpoints, site_positions
from helpers import example
from test_observables_cpu import _bcc_afm, _bcc_shells

pytestmark = pytest.mark.gpu

AXES = np.array([[1.0, 0.0, 0.0], [-1.0, 0.0, 0.0]])
COEFF = np.array([1, -1])


def _engine(h, tems, kernel, axes=AXES, coeff=COEFF):
    e = Engine(h.n, h.num_atoms, h.supercell, len(tems))
    e.upload(h)
    e.set_observables(order_axes=axes, staggered_coeff=coeff)
    e.set_temperatures(tems)
    e.set_sweep_kernel(kernel)
    return e


def _binning(series, levels, steps):
    """mcarlo.F90:548-590 and :635-656 for one column of per-measurement values."""
    out = []
    for lv in levels:
        blk = 2 ** lv
        ls, bn = 0.0, 0.0
        for k, v in enumerate(series, start=1):
            ls += v
            if k % blk == 0:
                ls /= blk
                bn += ls * ls
                ls = 0.0
        m_l = steps // blk
        v = (sum(series) - ls) / blk / m_l
        out.append((bn / m_l - v * v) / (m_l - 1))
    return np.array(out)


def _cells(h, s, axes, coeff):
    """Per unit cell: signed sum of s.a and |sum c s| (Pm_get)."""
    na = h.num_atoms
    c = s.reshape(-1, na, 3)
    op = np.einsum("kac,ac->k", c, axes)
    sm = np.linalg.norm(np.einsum("kac,a->kc", c, coeff.astype(float)), axis=1)
    return op, sm


def _bins(v, m_min, m_max, nf):
    x = (v - m_min) / (m_max - m_min) * (nf - 1)
    b = np.clip(np.floor(x + 0.5).astype(int) + 1, 1, nf)
    edge = np.abs(x - np.floor(x) - 0.5) < 1e-4   # FP32 may land on either side
    return b, edge


@pytest.mark.parametrize("kernel", ["ell", "cluster", "tile"])
def test_measurements_equal_the_oracle_on_the_gpu_spins(kernel):
    inp = _bcc_afm(L=4, tems=(3.0, 6.0, 10.0, 20.0, 3.0, 6.0, 10.0, 20.0))
    h = build_hamiltonian(inp)
    H = O.Ham(h)
    tems = np.array(inp.tems)
    R, K, levels = len(tems), 48, [1, 2, 3]
    nf = H.num_freq()
    m_max = float(np.abs(h.mag[:h.num_atoms]).sum())
    ncell = h.n // h.num_atoms
    host = np.zeros((R, 6))
    ser = np.zeros((R, K, 2))
    hop = np.zeros((R, nf), dtype=np.int64)
    hsm = np.zeros((R, nf), dtype=np.int64)
    slack = np.zeros(R, dtype=np.int64)
    with _engine(h, tems, kernel) as e:
        assert e.sweep_kernel()[0] == kernel
        e.init_spins("rand", seed=5)
        e.begin(e.schedule(20, K, 2, seed=77, binning_level=levels))
        for k in range(K):
            e.advance(1)
            S = e.get_spins()
            for t in range(R):
                s = S[t].reshape(-1)
                o2 = H.orderparam2(AXES, s)
                q2 = H.staggered2(COEFF.astype(float), s)
                host[t] += [np.sqrt(o2), o2, o2 * o2, np.sqrt(q2), q2, q2 * q2]
                ser[t, k] = [np.sqrt(o2), np.sqrt(q2)]
                op, sm = _cells(h, S[t], AXES, COEFF)
                for v, hist in ((op, hop), (sm, hsm)):
                    b, edge = _bins(v, -m_max, m_max, nf)
                    np.add.at(hist[t], b - 1, 1)
                    slack[t] += int(edge.sum())
        r = e.collect()
    assert np.allclose(r["obs_data"], host / K, rtol=1e-5, atol=1e-6)
    for t in range(R):
        for c in range(2):
            want = _binning(list(ser[t, :, c]), levels, K)
            assert np.allclose(r["obs_binning"][t, :, c], want, rtol=1e-4, atol=1e-12), (t, c)
    for got, want in ((r["pm_op"], hop), (r["pm_sm"], hsm)):
        cnt = np.rint(got * K * ncell / 100.0).astype(np.int64)
        assert np.array_equal(cnt.sum(axis=1), np.full(R, K * ncell))
        # bins agree except for cells within FP32 rounding of a bin edge
        assert np.all(np.abs(cnt - want).sum(axis=1) <= 2 * slack), (np.abs(cnt - want).sum(axis=1), slack)


@pytest.mark.parametrize("pt", [False, True])
def test_cluster_kernel_measurements_match_ell(pt):
    inp = _bcc_afm(L=8, tems=tuple(np.geomspace(4.0, 40.0, 8)))
    h = build_hamiltonian(inp)
    res = {}
    for kernel in ("ell", "cluster"):
        with _engine(h, inp.tems, kernel) as e:
            e.init_spins("ferro")
            res[kernel] = e.run(30, 200, 2, pt=pt, pt_steps_swap=5, seed=41, binning_level=[1, 2, 3])
    a, b = res["ell"], res["cluster"]
    assert np.array_equal(a["rejected"], b["rejected"])
    assert np.array_equal(a["map"], b["map"])
    assert np.allclose(a["obs_data"], b["obs_data"], rtol=1e-5, atol=1e-7)
    assert np.allclose(a["obs_binning"], b["obs_binning"], rtol=1e-3, atol=1e-12)
    # the same explicitly rounded FP32 sums per cell: identical histograms
    assert np.array_equal(a["pm_op"], b["pm_op"])
    assert np.array_equal(a["pm_sm"], b["pm_sm"])


@pytest.mark.parametrize("kernel", ["ell", "cluster"])
def test_unit_coefficients_repeat_the_magnetisation(kernel):
    inp = _bcc_afm(L=4, tems=(5.0, 30.0))
    h = build_hamiltonian(inp)
    with _engine(h, inp.tems, kernel, axes=None, coeff=np.array([1, 1])) as e:
        e.init_spins("rand", seed=3)
        r = e.run(20, 300, 1, seed=8, binning_level=[1, 2])
    assert r["pm_op"] is None
    assert np.array_equal(r["pm_sm"], r["pm"])
    assert np.allclose(r["obs_data"][:, 3:6], r["data"][:, 3:6], rtol=1e-5, atol=1e-7)
    assert np.allclose(r["obs_binning"][:, :, 1], r["binning"][:, :, 1], rtol=1e-3, atol=1e-12)


def test_staggered_and_order_parameter_match_reference_algorithm():
    """GPU colour-class chains against the oracle's typewriter chains: the
    means of <|OP|> and <SM> over chains agree within 3 sigma, sigma from the
    binning variances (largest over block sizes 2^4..2^7)."""
    tems = [8.0, 16.0, 30.0]
    inp = _bcc_afm(L=4, tems=tems)
    h = build_hamiltonian(inp)
    levels = list(range(1, 8))
    warm, steps, copies, chains = 2000, 20000, 4, 2
    rt = np.repeat(np.asarray(tems), copies)
    with _engine(h, rt, "auto") as e:
        e.init_spins("ferro")
        r = e.run(warm, steps, 1, seed=99, binning_level=levels)
    g = r["obs_data"].reshape(len(tems), copies, 6)[:, :, [0, 3]]
    gs = np.sqrt(np.max(np.maximum(r["obs_binning"].reshape(len(tems), copies, len(levels), 2)[:, :, 3:], 0),
                        axis=2))
    H = O.Ham(h)
    for t, T in enumerate(tems):
        od, osig = [], []
        for c in range(chains):
            s = np.zeros((h.n, 3)); s[:, 2] = 1.0
            o = H.mcarlo(O.MT(500 + 10 * c + t), 1.0 / T, s, warm, steps, 1, binning_level=levels,
                         want_pm=False, op_axes=AXES, st_coeff=COEFF.astype(float))
            od.append(o["obs_data"][0, [0, 3]] / steps)
            osig.append(np.sqrt(np.max(np.maximum(o["obs_binning"][0][3:], 0), axis=0)))
        gm, gsd = g[t].mean(axis=0), np.sqrt((gs[t] ** 2).sum(axis=0)) / copies
        om, osd = np.mean(od, axis=0), np.sqrt((np.array(osig) ** 2).sum(axis=0)) / chains
        sig = np.sqrt(gsd ** 2 + osd ** 2)
        assert np.all(np.abs(gm - om) <= 3.0 * sig), (T, gm, om, sig)


def test_host_driver_writes_order_parameter_files(tmp_path):
    inp, _ = example("ex03_fef3")
    inp.steps_warmup, inp.steps_mc, inp.steps_measure = 50, 200, 1
    inp.lstaggered = True
    inp.staggered_coeff = np.array([1, -1, 1, -1])
    inp.lbinerror = True
    inp.binning_level = [1, 2, 3]
    r = mc.run(inp, seed=5, outdir=str(tmp_path))
    base = os.path.join(str(tmp_path), inp.seedname)
    for suffix, ncol in (("_op.dat", 4), ("_staggered.dat", 4)):
        rows = [l.split() for l in open(base + suffix) if l.strip() and not l.lstrip().startswith("#")]
        assert len(rows) == len(inp.tems) and all(len(x) == ncol for x in rows)
        assert abs(float(rows[0][0]) - inp.tems[0]) < 1e-4
    pm_rows = [l.split() for l in open(base + "_pm.dat") if l.strip() and not l.lstrip().startswith("#")]
    assert all(len(x) == 4 for x in pm_rows)
    bin_rows = [l.split() for l in open(base + "_binerror.dat") if l.strip() and not l.lstrip().startswith("#")]
    assert all(len(x) == 5 for x in bin_rows) and len(bin_rows) == 3 * len(inp.tems)
    # the file's OP column is the collected <|OP|>
    op = [float(x[1]) for x in [l.split() for l in open(base + "_op.dat") if not l.lstrip().startswith("#")]]
    assert np.allclose(op, r.res["obs_data"][:, 0], rtol=1e-7)


@pytest.mark.parametrize("kernel", ["ell", "cluster", "tile"])
def test_spin_correlations_equal_the_oracle_on_the_gpu_spins(kernel):
    tems = (2.0, 5.0, 12.0, 40.0)
    inp = _bcc_shells(L=4, tems=tems)
    h = build_hamiltonian(inp)
    sh = build_shells(inp)
    H = O.Ham(h)
    R, K = len(tems), 24
    acc = np.zeros((3, R, 2, 2, 2))
    with Engine(h.n, h.num_atoms, h.supercell, R) as e:
        e.upload(h)
        e.set_spin_correlation(sh)
        e.set_temperatures(tems)
        e.set_sweep_kernel(kernel)
        assert e.sweep_kernel()[0] == kernel
        e.init_spins("rand", seed=2)
        e.begin(e.schedule(10, K, 1, seed=5))
        for _ in range(K):
            e.advance(1)
            S = e.get_spins()
            for t in range(R):
                sc, sa, st = H.spincorr(sh, S[t].reshape(-1))
                acc[0, t] += sc; acc[1, t] += sa; acc[2, t] += st
        r = e.collect()
    for k, name in enumerate(("spincorr", "spincorr_abs", "spincorr_tot")):
        want = acc[k] / K / h.n
        assert np.allclose(r[name], want, rtol=1e-5, atol=1e-7), name


@pytest.mark.parametrize("pt", [False, True])
def test_cluster_kernel_spin_correlations_match_ell(pt):
    inp = _bcc_shells(L=8, tems=tuple(np.geomspace(3.0, 30.0, 6)))
    h = build_hamiltonian(inp)
    sh = build_shells(inp)
    res = {}
    for kernel in ("ell", "cluster"):
        with Engine(h.n, h.num_atoms, h.supercell, len(inp.tems)) as e:
            e.upload(h)
            e.set_spin_correlation(sh)
            e.set_temperatures(inp.tems)
            e.set_sweep_kernel(kernel)
            e.init_spins("ferro")
            res[kernel] = e.run(20, 60, 2, pt=pt, pt_steps_swap=4, seed=13)
    a, b = res["ell"], res["cluster"]
    assert np.array_equal(a["rejected"], b["rejected"])
    for name in ("spincorr", "spincorr_abs", "spincorr_tot"):
        assert np.allclose(a[name], b[name], rtol=1e-5, atol=1e-7), name


def test_host_driver_writes_spin_correlation_file(tmp_path):
    inp, g = example("ex05_snwo")
    inp.steps_warmup, inp.steps_mc, inp.steps_measure = 50, 100, 1
    mc.run(inp, seed=3, outdir=str(tmp_path))
    rows = [l.split() for l in open(os.path.join(str(tmp_path), inp.seedname + "_spincorr.dat"))
            if l.strip() and not l.lstrip().startswith("#")]
    assert len(rows) == 4 * len(inp.tems)
    assert rows[0][2] == "Ni" and rows[3][1] == "4"
    # at the lowest temperature shells 3 and 4 are antiferromagnetic, as in
    # the reference's file
    assert float(rows[2][6]) < -0.5 and float(rows[3][6]) < -0.5


@pytest.mark.parametrize("pt", [False, True])
def test_energy_series_files(tmp_path, monkeypatch, pt):
    inp = _bcc_afm(L=4, tems=(3.0, 6.0, 12.0, 24.0))
    inp.steps_warmup, inp.steps_mc, inp.steps_measure = 20, 47, 1
    inp.pt, inp.pt_steps_swap = pt, 5
    inp.energy_write = True
    texts = []
    for budget, sub in ((1 << 28, "a"), (16 * 4 * 5 * 3, "b")):    # one chunk / chunks of 3 units
        monkeypatch.setattr(mc, "SERIES_BYTES", budget)
        r = mc.run(inp, seed=11, outdir=str(tmp_path / sub))
        texts.append([open(os.path.join(str(tmp_path / sub), "bcc_energy-T%03d.dat" % (t + 1))).read().splitlines()[1:]
                      for t in range(4)])
        nsteps = 50 if pt else 47
        for t in range(4):
            rows = texts[-1][t][2:]
            assert int(texts[-1][t][1]) == nsteps and len(rows) == nsteps
            assert [int(x.split()[0]) for x in rows] == list(range(1, nsteps + 1))
            # the last row is the final running energy per site
            assert float(rows[-1].split()[1]) == pytest.approx(r.res["energy"][t, 1] / r.ham.n, rel=1e-7)
    assert texts[0] == texts[1]


@pytest.mark.parametrize("kernel", ["ell", "cluster", "tile"])
def test_structure_factor_equals_the_oracle_on_the_gpu_spins(kernel):
    tems = (2.0, 6.0, 15.0, 40.0, 3.0)
    inp = _bcc_afm(L=4, tems=tems,
                   extra="sfactor = .true.\nsfactor_2dqmesh = 6 5\nsfactor_steps_measure = 3\n"
                         "sfactor_corner = -0.5 0 0.25\nsfactor_q1 = 2 2 0\nsfactor_q2 = 0 0 1.5\n"
                         "sfactor_polar = 0 1 1")
    h = build_hamiltonian(inp)
    H = O.Ham(h)
    q = sfactor_qpoints(inp)
    pos = site_positions(inp)
    R, K, every = len(tems), 13, 3
    want = np.zeros((R, q.shape[0], 3))
    with Engine(h.n, h.num_atoms, h.supercell, R) as e:
        e.upload(h)
        e.set_structure_factor(q, inp.sfactor_polar, every, inp.real_lattice, pos)
        e.set_temperatures(tems)
        e.set_sweep_kernel(kernel)
        assert e.sweep_kernel()[0] == kernel
        e.init_spins("rand", seed=8)
        e.begin(e.schedule(10, K, 1, seed=6))
        for k in range(1, K + 1):
            e.advance(1)
            if k % every == 0:
                S = e.get_spins()
                for t in range(R):
                    H.structure_factor(pos, q, inp.sfactor_polar, S[t].reshape(-1), want[t])
        r = e.collect()
    assert r["sfactor_count"] == K // every
    want /= h.n * (K // every)
    scale = want[..., 0].max()
    assert np.allclose(r["sfactor"], want, rtol=1e-4, atol=2e-5 * scale)


def test_host_driver_writes_structure_factor_files(tmp_path):
    inp = _bcc_afm(L=4, tems=(2.0, 30.0), extra="sfactor = .true.\nsfactor_2dqmesh = 4 4\nsfactor_steps_measure = 5")
    inp.steps_warmup, inp.steps_mc = 200, 100
    r = mc.run(inp, seed=2, outdir=str(tmp_path))
    rows = [l.split() for l in open(os.path.join(str(tmp_path), "bcc_sf-T001.dat"))]
    assert len(rows) == 25 and all(len(x) == 3 for x in rows)
    assert r.res["sfactor_count"] == 20
    # the antiferromagnetic Bragg peak at q = 2 pi (1, 0, 0) lies in the
    # default (h0l) plane: ordered at 2 K, not at 30 K
    assert r.res["sfactor"][0, :, 0].max() > r.res["sfactor"][1, :, 0].max()
