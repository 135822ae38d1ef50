"""Pins the FP64 oracle against the reference's own known answers.

The reference has no unit tests; its example runs are the known answers:
* seed-exact replay: each example prints the MT19937 seed of every MPI rank,
  so the first temperature of a rank (ferro start, typewriter order) can be
  replayed update by update and must give the printed accept/reject counts,
  the energy triple and the ``_mc.dat`` row, and the final spins of the
  ``_sconfig.dat`` file (mcarlo.F90:496-733); where the example measured the
  order parameter, also its ``_op.dat`` row and the P(M) / P(OP) columns of
  ``_pm.dat`` (orderparam_get, Pm_get: get_quant.F90:396-493); where it
  measured spin correlations, its ``_spincorr.dat`` rows (spincorr_get,
  get_quant.F90:495-540, over the shells of jij.F90:449-503);
* energy fixtures: the final spins of every temperature and the printed
  "Final Energy by direct calculations" (energy_get, get_quant.F90:186-261);
* MT19937 (mtprng.f90) against numpy's MT19937 for non-negative seeds, and
  Philox4x32-10 against the Random123 known-answer vectors;
* byte compatibility of the output writers: the replayed numbers rendered by
  espins_gb300.writers give the reference's own lines character for
  character -- the _mc.dat row (format 125, mcarlo.F90:854), the .mcout
  summary block (mcarlo.F90:736-753), the _sconfig.dat header and spin block
  (mcarlo.F90:112-114,813-816) and the _pm.dat block (mcarlo.F90:784-811);
  read_sconfig (get_quant.F90:543-598) reads the reference's file back.
"""
import json
import os

import numpy as np
import pytest

import oracle as O
from espins_gb300 import writers as W
from espins_gb300.mcin import K_B, read_mcin
from espins_gb300.tables import build_hamiltonian, build_shells


def _load(golden_dir, name, nodes=4):
    inp = read_mcin(os.path.join(golden_dir, name + ".mcin"), num_nodes=nodes)
    with open(os.path.join(golden_dir, name + "_golden.json")) as fh:
        g = json.load(fh)
    return inp, g


def test_mt19937_matches_numpy_for_nonnegative_seeds():
    for seed in (0, 1, 4357, 216157685, 2147483647):
        mt = O.MT(seed)
        rs = np.random.RandomState(seed)
        ref = rs.randint(0, 2 ** 32, size=700, dtype=np.uint64)
        got = [mt.u32() for _ in range(700)]
        assert got == [int(x) for x in ref]


def test_mt19937_negative_seed_differs_from_uint32_init():
    # mtprng_init keeps the sign-extended seed in a 64-bit word and shifts it
    # logically, so a negative seed is NOT init_genrand(uint32(seed)).
    seed = -923138203
    mt = O.MT(seed)
    rs = np.random.RandomState(seed & 0xFFFFFFFF)
    assert [mt.u32() for _ in range(5)] != [int(x) for x in rs.randint(0, 2 ** 32, size=5, dtype=np.uint64)]


@pytest.mark.parametrize("ctr,key,expect", [
    ([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
    ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
    ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
     [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
])
def test_philox_known_answers(ctr, key, expect):
    assert [int(x) for x in O.philox4x32_10(ctr, key)] == expect


@pytest.mark.parametrize("name", ["ex01_cubic", "ex02_cubic_pt", "ex03_fef3", "ex04_bmno_mc", "ex05_snwo"])
def test_table_builders_agree(golden_dir, name):
    """Product pair expansion (espins_gb300.tables) == oracle restatement, bit for bit."""
    inp, _ = _load(golden_dir, name, nodes=32 if name.startswith(("ex02", "ex04")) else 4)
    h = build_hamiltonian(inp)
    blocks = [(inp.jij, inp.jij.value / K_B, h.jij)]
    if h.bij is not None:
        blocks.append((inp.bij, inp.bij.value / K_B, h.bij))
    if h.dij is not None:
        blocks.append((inp.dij, inp.dij_vectors_cart * (inp.dij.value / K_B)[:, None], h.dij))
    for blk, vals, tab in blocks:
        nn, nb, val = O.build_ell(inp.num_atoms, inp.atoms_frac, inp.mag_cell, inp.supercell_size,
                                  inp.boundary_open, blk.f1, blk.f2, vals)
        assert np.array_equal(nn, tab.nn)
        assert np.array_equal(nb, tab.nb)
        assert np.array_equal(val, tab.val)


def test_table_builders_agree_open_boundary(golden_dir):
    inp, _ = _load(golden_dir, "ex03_fef3")
    inp.boundary_open = True
    h = build_hamiltonian(inp)
    nn, nb, val = O.build_ell(inp.num_atoms, inp.atoms_frac, inp.mag_cell, inp.supercell_size,
                              True, inp.jij.f1, inp.jij.f2, inp.jij.value / K_B)
    assert np.array_equal(nn, h.jij.nn) and np.array_equal(nb, h.jij.nb) and np.array_equal(val, h.jij.val)
    assert nn.min() < nn.max()  # surface sites lost bonds


@pytest.mark.parametrize("name", ["ex01_cubic", "ex02_cubic_pt", "ex03_fef3", "ex05_snwo"])
def test_energy_of_reference_final_configurations(golden_dir, name):
    """energy_get on the printed final spins == printed direct energy (7 digits)."""
    inp, g = _load(golden_dir, name, nodes=32 if name.startswith("ex02") else 4)
    h = build_hamiltonian(inp)
    H = O.Ham(h)
    z = np.load(os.path.join(golden_dir, name + "_sconfig.npz"))
    rows = {round(r["T"], 4): r for r in g["rows"]}
    for T, s in zip(z["temps"], z["spins"]):
        e = H.energy(s.reshape(-1))
        ref = rows[round(float(T), 4)]["E_direct"]
        # 7 printed digits, spins rounded to 6 decimals
        assert abs(e - ref) <= 2e-6 * abs(ref) + 1e-3, (T, e, ref)


def _e8(x):
    """x as Fortran's E15.8 prints it (8 significant digits)."""
    return float("%.7E" % x)


def _file_lines(path):
    with open(path) as fh:
        return fh.read().splitlines()


def _replay(golden_dir, name, rank, check_mcdat=True, check_obs=False, check_spincorr=False, tmp_path=None):
    inp, g = _load(golden_dir, name)
    h = build_hamiltonian(inp)
    H = O.Ham(h)
    nodes = len(g["seeds"])
    t_index = rank  # first local temperature of rank r is global index r (mcarlo.F90:500)
    T = inp.tems[t_index]
    s = np.zeros((h.n, 3))
    s[:, 2] = h.mag                     # initial_sconfig = ferro
    mt = O.MT(g["seeds"][rank])
    obs = {"op_axes": inp.orderparam_axes_cart} if check_obs else {}
    if check_spincorr:
        obs["shells"] = build_shells(inp)
    r = H.mcarlo(mt, 1.0 / T, s, inp.steps_warmup, inp.steps_mc, inp.steps_measure,
                 binning_level=[1, 2, 3, 4, 5], **obs)
    row = g["rows"][t_index]
    assert abs(row["T"] - T) < 1e-4
    assert r["steps_tot"] == [row["warmup"][0], row["mc"][0]]
    assert r["rejected"] == [row["warmup"][1], row["mc"][1]]
    for k, v in zip(("E_init", "E_add", "E_direct"), r["energy"]):
        assert abs(v - row[k]) <= 6e-7 * abs(row[k]), (k, v, row[k])
    z = np.load(os.path.join(golden_dir, name + "_sconfig.npz"))
    assert np.max(np.abs(s - z["spins"][t_index])) <= 5.01e-7
    if check_mcdat:
        N = h.n
        d = r["data"] / inp.steps_mc
        beta = 1.0 / T
        C = beta * beta * (d[1] - d[0] ** 2) / N
        chi = beta * (d[4] - d[3] ** 2) * N
        UE = 1.0 - (1.0 / 3.0) * (d[2] / d[1] ** 2)
        UM = 1.0 - (1.0 / 3.0) * (d[5] / d[4] ** 2)
        got = [T, d[3], d[0] / N, C, chi, UE, UM]
        ref = g["mc_dat"][t_index]
        for a, b in zip(got[1:], ref[1:]):
            # Fortran E15.8 keeps 8 significant digits
            assert float("%.7E" % a) == pytest.approx(b, rel=1e-12, abs=1e-300)
        # the writers render the same numbers as the reference's lines
        assert W.mc_dat_row(T, d, N) == g["mc_dat_lines"][t_index]
        res = {"steps_mc_eff": inp.steps_mc, "steps_tot": r["steps_tot"], "rejected": [r["rejected"]],
               "energy": [r["energy"]], "data": [d]}
        assert W.mcout_block([T], res, N, False).splitlines() == g["mcout_blocks"][t_index]
        if tmp_path is not None and "sconfig_lines" in g and t_index == 0:
            allspins = np.repeat(s[None], inp.tems_num, axis=0)
            path = os.path.join(str(tmp_path), "x_sconfig.dat")
            W.write_sconfig(path, inp.supercell_size, inp.tems, allspins)
            lines = _file_lines(path)
            assert lines[0].startswith(" Created on ")
            assert lines[1:1 + len(g["sconfig_lines"])] == g["sconfig_lines"]
    if check_obs:
        N = h.n
        beta = 1.0 / T
        normalize = 1.0 / inp.steps_mc
        d = r["obs_data"][0] * normalize
        sus = beta * (d[1] - d[0] ** 2) * N
        U = 1.0 - (1.0 / 3.0) * (d[2] / d[1] ** 2)
        ref = g["op_dat"][t_index]
        assert abs(ref[0] - T) < 1e-4
        for a, b in zip([d[0], sus, U], ref[1:]):
            assert _e8(a) == pytest.approx(b, rel=1e-12, abs=1e-300)
        # _pm.dat: global_pm * normalize / num_supercell (mcarlo.F90:713-715)
        rows = np.array(g["pm_dat"]["%.4f" % T])
        ncell = N // h.num_atoms
        pm = r["pm"] * normalize / ncell
        pop = r["pm_op"][0] * normalize / ncell
        assert rows.shape == (pm.size, 3)
        for f in range(pm.size):
            assert _e8(pm[f]) == pytest.approx(rows[f, 1], rel=1e-12, abs=1e-300), f
            assert _e8(pop[f]) == pytest.approx(rows[f, 2], rel=1e-12, abs=1e-300), f
        if tmp_path is not None:
            m_max = float(np.abs(inp.mag_cell).sum())
            path = os.path.join(str(tmp_path), "x_pm.dat")
            W.write_pm_dat(path, [T], pm[None], -m_max, m_max, pm_op=pop[None], pt=False)
            lines = _file_lines(path)
            assert lines[0].startswith(" #written on ")
            assert lines[1:4] == g["pm_dat_head"]
            assert lines[4:] == g["pm_dat_lines"]["%.4f" % T]
    if check_spincorr:
        # global_spincorr * normalize / N (mcarlo.F90:717-723), printed f12.9
        normalize = 1.0 / inp.steps_mc
        got = {k: r[k][0] * normalize / h.n for k in ("spincorr", "spincorr_abs", "spincorr_tot")}
        rows = [x for x in g["spincorr_dat"] if abs(x[0] - T) < 1e-4]
        assert len(rows) == got["spincorr"].size
        for x in rows:
            sh, a, b = x[1] - 1, x[2] - 1, x[3] - 1
            for k, want in zip(("spincorr", "spincorr_abs", "spincorr_tot"), x[4:7]):
                assert float("%.9f" % got[k][sh, a, b]) == pytest.approx(want, abs=1e-15), (k, x)
    return r


def test_seed_exact_replay_ex01_negative_seed(golden_dir, tmp_path):
    _replay(golden_dir, "ex01_cubic", rank=0, tmp_path=tmp_path)


def test_seed_exact_replay_ex01_positive_seed(golden_dir):
    _replay(golden_dir, "ex01_cubic", rank=3)


def test_seed_exact_replay_ex05_biquadratic_singleion(golden_dir):
    _replay(golden_dir, "ex05_snwo", rank=0, check_mcdat=True, check_spincorr=True)


def test_seed_exact_replay_ex03_biquadratic_dm(golden_dir, tmp_path):
    _replay(golden_dir, "ex03_fef3", rank=1, check_mcdat=True, check_obs=True, tmp_path=tmp_path)


def test_read_sconfig_reads_the_reference_file(golden_dir, tmp_path):
    """read_sconfig on the reference's _sconfig.dat text (header and the first
    temperature block of example01): spins normalised to unit length, and the
    reference's error checks (mcarlo_read_sconfig, get_quant.F90:543-598)."""
    _, g = _load(golden_dir, "ex01_cubic")
    lines = list(g["sconfig_lines"])
    n = int(lines[1].split()[0])
    lines[1] = f"{n:6d}{1:6d}"            # the fixture keeps one temperature block
    path = os.path.join(str(tmp_path), "ref_sconfig.dat")
    with open(path, "w") as fh:
        fh.write(" Created on  1Dec2019 at 16:53:37 \n" + "\n".join(lines) + "\n")
    z = np.load(os.path.join(golden_dir, "ex01_cubic_sconfig.npz"))
    got = W.read_sconfig(path, n, [25.0])
    want = z["spins"][0] / np.linalg.norm(z["spins"][0], axis=1, keepdims=True)
    assert got.shape == (1, n, 3)
    assert np.allclose(got[0], want, atol=1e-15)
    with pytest.raises(ValueError, match="Wrong matrix size"):
        W.read_sconfig(path, n + 1, [25.0])
    with pytest.raises(ValueError, match="Wrong temperature number"):
        W.read_sconfig(path, n, [25.0, 30.0])
    with pytest.raises(ValueError, match="Mismatch in temperatures"):
        W.read_sconfig(path, n, [25.01])
    lines[3] = "    0.000000    0.000000    0.000000"
    with open(path, "w") as fh:
        fh.write(" Created\n" + "\n".join(lines) + "\n")
    with pytest.raises(ValueError, match="zero"):
        W.read_sconfig(path, n, [25.0])


def test_pt_mcout_block_layout(golden_dir):
    """The parallel-tempering summary (pt.F90:983-1021) rendered from
    example02's printed numbers reproduces its lines: the final swap table
    (format 128) and, per temperature, the MCARLO line and the energy triple
    marked ENERGY3.  (Delta E / Delta M need the unprinted accumulators.)"""
    inp, g = _load(golden_dir, "ex02_cubic_pt", nodes=32)
    tems = [r["T"] for r in g["rows"]]
    R = len(tems)
    sw = g["swaps"]
    res = {
        "steps_mc_eff": inp.steps_mc,
        "steps_tot": [0, g["rows"][0]["mc"][0]],
        "rejected": [[0, r["mc"][1]] for r in g["rows"]],
        "energy": [[r["E_init"], r["E_add"], r["E_direct"]] for r in g["rows"]],
        "data": [[0.0] * 6 for _ in range(R)],
        "num_swaps": [[row[2], row[4]] for row in sw],
        "map": [1 + min(range(R), key=lambda k: abs(tems[k] - row[1])) for row in sw],
    }
    lines = W.mcout_block(tems, res, 2744, True).splitlines()
    n_swap = len(g["swap_lines"])
    assert lines[1:1 + n_swap] == g["swap_lines"]
    blocks = lines[1 + n_swap + 4:]
    for t, ref in enumerate(g["mcout_blocks"]):
        got = blocks[7 * t: 7 * t + 7]
        assert got[:4] == ref[:4], t
