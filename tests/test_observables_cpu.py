"""The order parameter and the staggered magnetisation on the CPU side:

* the oracle's orderparam_get / staggered_get / Pm_get restatement against
  identities that hold for any configuration (all staggered coefficients +1
  give the magnetisation; axes along z give m_z), and over a whole chain
  (the staggered columns of a run with +1 coefficients equal its |m| columns);
* the writers' format 126 against rows of the reference's own _op.dat;
* the input parser's staggered_m_coeff rules (parameters.F90:450-463).
The oracle's order parameter is pinned to the reference's ex03 _op.dat row and
P(OP) column by the seed-exact replay in test_oracle_golden.py.
"""
import numpy as np
import pytest

import oracle as O
from espins_gb300 import writers as W
from espins_gb300.mcin import McinError, parse_mcin
from espins_gb300.tables import build_hamiltonian
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
