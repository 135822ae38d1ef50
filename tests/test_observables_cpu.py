"""The order parameter, the staggered magnetisation and the spin correlations
on the CPU side:

* the oracle's orderparam_get / staggered_get / Pm_get restatement against
  identities that hold for any configuration (all staggered coefficients +1
  give the magnetisation; axes along z give m_z), and over a whole chain
  (the staggered columns of a run with +1 coefficients equal its |m| columns);
* the writers' format 126 and the _spincorr.dat row format against rows of
  the reference's own files;
* the neighbour shells of spincorr_get (jij.F90:449-503) and the oracle's
  spincorr_get on ordered states;
* the input parser's staggered_m_coeff rules (parameters.F90:450-463).
The oracle's order parameter is pinned to the reference's ex03 _op.dat row and
P(OP) column, and its spin correlations to the ex05 _spincorr.dat rows, by the
seed-exact replays in test_oracle_golden.py.
"""
import numpy as np
import pytest

import oracle as O
from espins_gb300 import writers as W
from espins_gb300.mcin import McinError, parse_mcin
from espins_gb300.tables import build_hamiltonian, build_shells
from helpers import NN, example, sc_mcin


def _bcc_afm(L=4, tems=(6.0,), extra=""):
    """Two-atom simple-cubic cell of a bcc lattice, nearest neighbours
    antiferromagnetic between the two atoms."""
    lines = ["begin unit_cell_cart", "1 0 0", "0 1 0", "0 0 1", "end unit_cell_cart",
             "begin atoms_frac", "Fe 0 0 0 1.0", "Co 0.5 0.5 0.5 1.0", "end atoms_frac",
             f"supercell_size = {L} {L} {L}", "tems_mode = man", f"tems_num = {len(tems)}",
             "tems = " + " ".join(repr(float(t)) for t in tems),
             "steps_warmup = 10", "steps_mc = 100", "steps_measure = 1",
             "begin jij_parameters"]
    for dx in (0.5, -0.5):
        for dy in (0.5, -0.5):
            for dz in (0.5, -0.5):
                lines.append(f"f1=0,0,0:f2={dx},{dy},{dz}:jij=-0.002")
                lines.append(f"f1=0.5,0.5,0.5:f2={0.5 + dx},{0.5 + dy},{0.5 + dz}:jij=-0.002")
    lines.append("end jij_parameters")
    lines += [l for l in extra.splitlines() if l.strip()]
    return parse_mcin("\n".join(lines) + "\n", seedname="bcc")


def _bcc_shells(L=4, tems=(6.0,), j1=-0.002, j2=0.0003):
    """bcc as a two-species simple-cubic cell (Fe at the corner, Co at the
    centre) with spin-correlation shells: sh=1 the 8 Fe-Co neighbours, sh=2 the
    6 same-species neighbours."""
    lines = ["begin unit_cell_cart", "1 0 0", "0 1 0", "0 0 1", "end unit_cell_cart",
             "begin atoms_frac", "Fe 0 0 0 1.0", "Co 0.5 0.5 0.5 1.0", "end atoms_frac",
             f"supercell_size = {L} {L} {L}", "tems_mode = man", f"tems_num = {len(tems)}",
             "tems = " + " ".join(repr(float(t)) for t in tems),
             "steps_warmup = 10", "steps_mc = 100", "steps_measure = 1", "spin_correlation = .true.",
             "begin jij_parameters"]
    for c in ((0, 0, 0), (0.5, 0.5, 0.5)):
        for dx in (0.5, -0.5):
            for dy in (0.5, -0.5):
                for dz in (0.5, -0.5):
                    lines.append(f"f1={c[0]},{c[1]},{c[2]}:f2={c[0] + dx},{c[1] + dy},{c[2] + dz}:jij={j1}:sh=1")
        for o in NN:
            lines.append(f"f1={c[0]},{c[1]},{c[2]}:f2={c[0] + o[0]},{c[1] + o[1]},{c[2] + o[2]}:jij={j2}:sh=2")
    lines.append("end jij_parameters")
    return parse_mcin("\n".join(lines) + "\n", seedname="bccsc")


def _random_spins(h, seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=(h.n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True) * h.mag[:, None]


def test_staggered_with_unit_coefficients_is_the_magnetisation():
    inp = _bcc_afm()
    h = build_hamiltonian(inp)
    H = O.Ham(h)
    s = _random_spins(h, 1)
    assert H.staggered2(np.ones(2), s.reshape(-1)) == H.magnetization2(s.reshape(-1))
    pm = H.pm(s.reshape(-1))
    _, ps = H.pm_obs(s.reshape(-1), coeff=np.ones(2))
    assert np.array_equal(pm, ps)


def test_order_parameter_along_z_is_mz_and_staggered_flips_a_sublattice():
    inp = _bcc_afm()
    h = build_hamiltonian(inp)
    H = O.Ham(h)
    s = _random_spins(h, 2)
    ax = np.array([[0.0, 0.0, 1.0], [0.0, 0.0, 1.0]])
    mz = s[:, 2].sum() / h.n
    assert H.orderparam2(ax, s.reshape(-1)) == pytest.approx(mz * mz, rel=1e-13)
    # site j belongs to atom j % num_atoms of its cell
    c = np.array([1.0, -1.0])
    stag = (s * c[np.arange(h.n) % 2][:, None]).sum(axis=0) / h.n
    assert H.staggered2(c, s.reshape(-1)) == pytest.approx(stag @ stag, rel=1e-13)
    # the Neel state along x: SM = 1, OP with axes (x, -x) = 1
    neel = np.zeros((h.n, 3))
    neel[:, 0] = c[np.arange(h.n) % 2]
    assert H.staggered2(c, neel.reshape(-1)) == pytest.approx(1.0, abs=1e-14)
    assert H.orderparam2(np.array([[1.0, 0, 0], [-1.0, 0, 0]]), neel.reshape(-1)) == pytest.approx(1.0, abs=1e-14)
    # every cell of the Neel state sits in the top P(SM) bin and the P(OP) bin of +2
    po, ps = H.pm_obs(neel.reshape(-1), axes=np.array([[1.0, 0, 0], [-1.0, 0, 0]]), coeff=c)
    nf = H.num_freq()
    ncell = h.n // 2
    assert ps[nf - 1] == pytest.approx(100.0 * ncell) and ps.sum() == pytest.approx(100.0 * ncell)
    assert po[nf - 1] == pytest.approx(100.0 * ncell)


def test_chain_with_unit_coefficients_repeats_the_magnetisation_columns():
    inp = _bcc_afm(tems=(4.0,))
    h = build_hamiltonian(inp)
    H = O.Ham(h)
    s = np.zeros((h.n, 3))
    s[:, 2] = h.mag
    r = H.mcarlo(O.MT(7), 1.0 / 4.0, s, 20, 256, 1, binning_level=[1, 2, 3],
                 st_coeff=np.ones(2), op_axes=np.array([[0.0, 0.0, 1.0], [0.0, 0.0, 1.0]]))
    assert np.array_equal(r["obs_data"][0, 3:6], r["data"][3:6])
    assert np.array_equal(r["obs_binning"][0, :, 1], r["binning"][:, 1])
    assert np.array_equal(r["pm_st"][0], r["pm"])
    # |OP| with z axes is |m_z| <= |m|
    assert r["obs_data"][0, 0] <= r["data"][3] + 1e-12


def test_pt_chain_with_unit_coefficients_repeats_the_magnetisation_columns():
    inp = _bcc_afm(tems=(3.0, 5.0, 8.0))
    h = build_hamiltonian(inp)
    H = O.Ham(h)
    s = np.zeros((3, h.n, 3))
    s[:, :, 2] = 1.0
    r = H.pt(O.MT(9), [3.0, 5.0, 8.0], s.reshape(-1), 20, 120, 1, 5, binning_level=[1, 2],
             st_coeff=np.ones(2))
    assert np.array_equal(r["obs_data"][:, 3:6], r["data"][:, 3:6])
    assert np.array_equal(r["obs_binning"][:, :, 1], r["binning"][:, :, 1])
    assert np.array_equal(r["pm_st"], r["pm"])


def test_format_126_reproduces_reference_op_rows():
    _, g = example("ex03_fef3")
    for line, row in zip(g["op_dat_lines"], g["op_dat"]):
        assert W.format126(*row) == line


def test_staggered_coefficients_default_and_validation():
    inp = _bcc_afm()
    assert list(inp.staggered_coeff) == [1, 1]
    inp = _bcc_afm(extra="staggered_m = .true.\nstaggered_m_coeff = 1 -1")
    assert inp.lstaggered and list(inp.staggered_coeff) == [1, -1]
    with pytest.raises(McinError):
        _bcc_afm(extra="staggered_m = .true.\nstaggered_m_coeff = 1 2")
    # one atom per cell: staggered_m is switched off
    one = sc_mcin(4, [(1e-3, NN)], [5.0], extra="staggered_m = .true.")
    assert not one.lstaggered


def test_spincorr_row_format_reproduces_reference_rows():
    _, g = example("ex05_snwo")
    for row, line in zip(g["spincorr_dat"], g["spincorr_dat_lines"]):
        assert W.spincorr_row(row[0], row[1], "Ni", row[2], "Ni", row[3], *row[4:]) == line


def test_shell_tables():
    inp, _ = example("ex05_snwo")
    t = build_shells(inp)
    assert t.num_shells == 4 and t.num_species == 1
    assert [int(x) for x in t.nn[:, 0]] == [4, 8, 4, 2]
    assert np.all(t.nn == t.nn[:, :1])
    # periodic shells are symmetric: j in shell s of i <=> i in shell s of j
    for s_ in range(t.num_shells):
        pairs = {(i, int(t.nb[s_, k, i])) for i in range(t.kind.size) for k in range(t.nn[s_, i])}
        assert all((j, i) in pairs for i, j in pairs)
    b = build_shells(_bcc_shells())
    assert b.num_species == 2
    assert [int(x) for x in b.nn[:, 0]] == [8, 6]
    # shell_num_nbors_kind(s, a, b): species-a neighbours around the last site of species b
    assert b.count[0].tolist() == [[0, 8], [8, 0]] and b.count[1].tolist() == [[6, 0], [0, 6]]


def test_oracle_spincorr_on_ordered_states():
    inp = _bcc_shells()
    h = build_hamiltonian(inp)
    H = O.Ham(h)
    sh = build_shells(inp)
    ferro = np.zeros((h.n, 3)); ferro[:, 2] = 1.0
    sc, sa, st = H.spincorr(sh, ferro.reshape(-1))
    # every existing (shell, species pair) bin sums to its number of sites
    want = np.zeros((2, 2, 2))
    want[0, 0, 1] = want[0, 1, 0] = want[1, 0, 0] = want[1, 1, 1] = h.n // 2
    assert np.allclose(sc, want) and np.allclose(sa, want) and np.allclose(st, want)
    neel = ferro.copy(); neel[1::2, 2] = -1.0      # Co antiparallel to Fe
    sc, sa, st = H.spincorr(sh, neel.reshape(-1))
    assert np.allclose(sc[0], -want[0]) and np.allclose(sc[1], want[1])
    assert np.allclose(sa, want) and np.allclose(st, want)


def test_energy_series_files_format(tmp_path):
    """open_E_unit / write_E layout: name seed_energy-T###.dat, '# T =' line,
    the number of measurements, rows (I14,4x,E16.8) of E/N in order."""
    assert W.energy_series_name("fef3", 7) == "fef3_energy-T007.dat"
    assert W.energy_series_name("fef3", 123) == "fef3_energy-T123.dat"
    s = W.EnergySeries(str(tmp_path / "x"), [5.0, 12.5], 5, 4)
    s.append(np.array([[-4.0, 2.0], [-8.0, 6.0]]))
    s.append(np.array([[-2.0, 0.4]] * 3))
    s.close()
    lines = open(tmp_path / "x_energy-T002.dat").read().splitlines()
    assert lines[1] == "   # T =   12.5000"
    assert lines[2] == "   " + " " * 15 + "5"
    assert lines[3] == "             1      0.50000000E+00"
    assert lines[4] == "             2      0.15000000E+01"
    assert len(lines) == 8 and lines[7].startswith("             5")
    first = open(tmp_path / "x_energy-T001.dat").read().splitlines()
    assert first[3] == "             1     -0.10000000E+01"


def test_oracle_structure_factor_identities():
    """mcarlo_structure_factor on a ferromagnet along z: at a reciprocal lattice
    vector G along x every site adds in phase, F = N z (transverse to G), so
    S = N^2 and NSF = N (polarisation along z) or 0 (along x); q = 0 adds
    nothing; and the restatement equals a direct numpy evaluation."""
    from espins_gb300.tables import site_positions
    inp = sc_mcin(4, [(1e-3, NN)], [5.0])
    h = build_hamiltonian(inp)
    H = O.Ham(h)
    pos = site_positions(inp)
    ferro = np.zeros((h.n, 3)); ferro[:, 2] = 1.0
    G = 2 * np.pi * np.array([[1.0, 0, 0], [0, 0, 0], [0.37, 0.1, 0.0]])
    sz = H.structure_factor(pos, G, [0.0, 0.0, 1.0], ferro.reshape(-1))
    sx = H.structure_factor(pos, G, [1.0, 0.0, 0.0], ferro.reshape(-1))
    N = h.n
    assert np.allclose(sz[0], [N * N, 0.0, N * N]) and np.allclose(sx[0], [N * N, N * N, 0.0])
    assert np.all(sz[1] == 0.0)
    rng = np.random.default_rng(4)
    s = rng.normal(size=(N, 3)); s /= np.linalg.norm(s, axis=1, keepdims=True)
    p = np.array([0.3, -0.2, 0.9])
    got = H.structure_factor(pos, G, p, s.reshape(-1))
    for k, q in enumerate(G):
        if not q.any():
            continue
        ph = np.exp(1j * pos @ q)
        perp = s - np.outer(s @ q, q) / (q @ q)
        F = (perp * ph[:, None]).sum(axis=0)
        nsf = float(np.real(((perp @ p) * ph).sum())) / np.linalg.norm(p)
        f2 = float(np.sum(np.abs(F) ** 2))
        assert np.allclose(got[k], [f2, f2 - nsf ** 2, nsf ** 2], rtol=1e-10, atol=1e-9)


def test_sfactor_input_and_plane_coordinates():
    from espins_gb300.tables import sfactor_qpoints
    inp = sc_mcin(4, [(1e-3, NN)], [5.0], extra="sfactor = .true.\nsfactor_2dqmesh = 4 2\nsfactor_steps_measure = 10\n"
                                               "sfactor_q1 = 1 1 0\nsfactor_q2 = 0 0 2\nsfactor_polar = 0 0 1")
    assert inp.lsfactor and inp.lsfactor_polar and inp.sfactor_steps_measure == 10
    q = sfactor_qpoints(inp)
    assert q.shape == (15, 3)
    assert np.allclose(q[1], 2 * np.pi * np.array([0, 0, 1.0]))        # i = 0, j = 1 of 2
    assert np.allclose(q[3], 2 * np.pi * np.array([0.25, 0.25, 0.0]))  # i = 1, j = 0
    xy = W.sfactor_plane_coords(inp.sfactor_corner, inp.sfactor_q1, inp.sfactor_q2, inp.sfactor_2dqmesh)
    # q1 and q2 orthogonal: x along q1 (|q1| = 2 pi sqrt 2), y along q2 (|q2| = 4 pi)
    assert np.allclose(xy[3], (0.25 * 2 * np.pi * np.sqrt(2), 0.0))
    assert np.allclose(xy[1], (0.0, 0.5 * 4 * np.pi))
    with pytest.raises(McinError):
        sc_mcin(4, [(1e-3, NN)], [5.0], extra="sfactor = .true.\nsfactor_q1 = 1 0 0\nsfactor_q2 = 2 0 0")
