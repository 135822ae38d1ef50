"""GPU parity of the hot-path kernels against the FP64 oracle (through the C ABI).

Tolerances (FP32 site fields, FP64 totals), the 1e-6 relative bar:
* local terms g_i, Q_i: |gpu - oracle| <= 1e-6 * sum_k(|J_ik|+|B_ik|+|D_ik|)
  (FIELD_RTOL; measured at most 3.9e-7)
* total energy:         |gpu - oracle| <= 1e-6 * sum of |coupling| (energy_scale;
  ENERGY_RTOL; measured at most 4.1e-8)
* one colour pass: every accept/reject decision equal to the oracle's except
  where |exp(-beta dE) - u| < 1e-4 (FP32 rounding of dE can flip those), and
  the new spins within 2e-6 of the oracle's FP64 trial spins.
"""
import ctypes

import numpy as np
import pytest

import oracle as O
from espins_gb300.lib import Engine
from espins_gb300.tables import build_hamiltonian
from helpers import (ENERGY_RTOL, FIELD_RTOL, N3, NN, NNN, energy_scale, example, example_spins, sc_mcin,
                     site_scale)

pytestmark = pytest.mark.gpu

EXAMPLES = ["ex01_cubic", "ex03_fef3", "ex05_snwo", "ex02_cubic_pt"]


def _engine(h, R, tems=None):
    e = Engine(h.n, h.num_atoms, h.supercell, R)
    e.upload(h)
    e.set_temperatures(np.linspace(5.0, 50.0, R) if tems is None else tems)
    return e


def _f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


@pytest.mark.parametrize("name", EXAMPLES)
def test_energy_matches_oracle_on_reference_configurations(name):
    inp, _ = example(name)
    h = build_hamiltonian(inp)
    temps, spins = example_spins(name)
    R = len(temps)
    H = O.Ham(h)
    with _engine(h, R, temps) as e:
        e.set_spins(spins)
        got = e.energy()
        ref = np.array([H.energy(_f32(s).reshape(-1)) for s in spins])
        tol = ENERGY_RTOL * energy_scale(h)
        print(f"\n{name}: energy error / scale {np.max(np.abs(got - ref)) / energy_scale(h):.2e}")
        assert np.max(np.abs(got - ref)) <= tol, (got - ref, tol)
        # running values were reset to the direct ones
        assert np.array_equal(e.running_energy(), got)
        m = e.running_magnetization()
        assert np.allclose(m, _f32(spins).sum(axis=1), atol=1e-6 * h.n)


@pytest.mark.parametrize("name", EXAMPLES)
def test_local_terms_match_oracle(name):
    inp, _ = example(name)
    h = build_hamiltonian(inp)
    temps, spins = example_spins(name)
    R = min(len(temps), 3)
    H = O.Ham(h)
    with _engine(h, R, temps[:R]) as e:
        e.set_spins(spins[:R])
        g, q = e.local_terms()
        sc = site_scale(h)[:, None]
        for t in range(R):
            gr, qr = H.local_terms(_f32(spins[t]).reshape(-1))
            eg, eq = np.max(np.abs(g[t] - gr) / sc), np.max(np.abs(q[t] - qr) / sc)
            print(f"\n{name}[{t}]: field error / site scale {eg:.2e}, quadratic form {eq:.2e}")
            assert eg <= FIELD_RTOL
            assert eq <= FIELD_RTOL


def _synthetic_cases():
    return {
        "sc_j1": (sc_mcin(6, [(1e-3, NN)], [3.0, 10.0, 30.0]), None),
        "sc_j1j2_bq_si": (sc_mcin(6, [(1e-3, NN), (-6e-4, NNN)], [2.0, 8.0, 30.0], bq=5e-5, si=2e-4), None),
        "sc_j123_dm_si": (sc_mcin(6, [(1e-3, NN), (3e-4, NNN), (-5e-5, N3)], [5.0, 20.0, 40.0], dm=1e-4, si=-3e-5), None),
    }


@pytest.mark.parametrize("case", ["sc_j1", "sc_j1j2_bq_si", "sc_j123_dm_si"])
@pytest.mark.parametrize("mode", [0, 1])
def test_single_colour_pass_matches_oracle(case, mode):
    inp, _ = _synthetic_cases()[case]
    h = build_hamiltonian(inp)
    R = len(inp.tems)
    H = O.Ham(h)
    rng = np.random.default_rng(7)
    v = rng.normal(size=(R, h.n, 3))
    spins = v / np.linalg.norm(v, axis=2, keepdims=True)
    seed, sweep, tilt = 0x1234ABCD5678, 17, 0.3
    with _engine(h, R, inp.tems) as e:
        e.set_spins(spins)
        colour, C = e.colouring()
        assert C >= 2
        for c in range(C):
            before = e.get_spins()
            e0 = e.running_energy()
            e.sweep_colour(c, sweep, seed, mode=mode, tilt=tilt)
            after = e.get_spins()
            e1 = e.running_energy()
            for t in range(R):
                s = before[t].reshape(-1).copy()
                rej, de_sum, acc, de = H.colour_pass_philox(colour, c, 1.0 / inp.tems[t], s, t, sweep, seed,
                                                            mode=mode, tilt=tilt)
                s = s.reshape(-1, 3)
                in_c = colour == c
                moved = np.any(after[t] != before[t], axis=1)
                # oracle decisions; flips allowed only at the acceptance threshold
                x = np.array([O.philox4x32_10([i, t, sweep, 0], [seed & 0xFFFFFFFF, seed >> 32])[2]
                              for i in range(h.n)])
                u = (x >> 8).astype(np.float64) / 16777216.0
                margin = np.abs(np.exp(-np.clip(de, -50, 50) / inp.tems[t]) - u)
                disagree = in_c & ((acc == 1) != moved) & ~((de > 0) & (margin < 1e-4))
                # a trial equal to the old spin cannot be seen as a move
                assert not np.any(disagree), np.nonzero(disagree)
                ok = in_c & (acc == 1) & moved
                assert np.max(np.abs(after[t][ok] - s[ok]), initial=0.0) <= 2e-6
                assert np.array_equal(after[t][~in_c], before[t][~in_c])
                assert abs((e1[t] - e0[t]) - de_sum) <= 1e-4 * (1 + abs(de_sum)) + 1e-5 * h.n


def test_running_energy_tracks_direct_energy_over_many_sweeps():
    inp, _ = _synthetic_cases()["sc_j123_dm_si"]
    h = build_hamiltonian(inp)
    R = len(inp.tems)
    with _engine(h, R, inp.tems) as e:
        e.init_spins("rand", seed=3)
        e.sweep(200, 0, seed=11)
        run = e.running_energy()
        m_run = e.running_magnetization()
        direct = e.energy()
        s = e.get_spins()
        assert np.max(np.abs(run - direct)) <= 1e-5 * energy_scale(h)
        assert np.allclose(m_run, s.sum(axis=1), atol=1e-4 * h.n)
        # every spin keeps its length
        assert np.allclose(np.linalg.norm(s, axis=2), 1.0, atol=2e-6)


def test_same_seed_same_trajectory():
    inp, _ = _synthetic_cases()["sc_j1j2_bq_si"]
    h = build_hamiltonian(inp)
    R = len(inp.tems)
    outs = []
    for _ in range(2):
        with _engine(h, R, inp.tems) as e:
            e.init_spins("ferro")
            e.sweep(50, 100, seed=99)
            outs.append(e.get_spins())
    assert np.array_equal(outs[0], outs[1])


def test_colouring_is_proper_and_minimal_on_lattices():
    for L, shells, expect in [(8, [(1e-3, NN)], 2), (8, [(1e-3, NN), (1e-4, NNN)], 4),
                              (8, [(1e-3, NN), (1e-4, NNN), (1e-5, N3)], 8)]:
        inp = sc_mcin(L, shells, [10.0])
        h = build_hamiltonian(inp)
        with _engine(h, 1, [10.0]) as e:
            col, C = e.colouring()
        assert C == expect
        for k in range(h.jij.maxnb):
            assert np.all(col[h.jij.nb[k]] != col)


def test_pt_swap_kernel_takes_the_host_protocol_decisions():
    """k_pt_swap == espins_gb300.distributed.swap_decisions on the same energies."""
    from espins_gb300 import distributed as D
    inp = sc_mcin(4, [(1e-3, NN)], list(np.geomspace(5.0, 40.0, 10)))
    h = build_hamiltonian(inp)
    R = len(inp.tems)
    rng = np.random.default_rng(3)
    seed = 0x5EED5EED12345
    with _engine(h, R, inp.tems) as e:
        for step in range(6):
            v = rng.normal(size=(R, h.n, 3))
            e.set_spins(v / np.linalg.norm(v, axis=2, keepdims=True))   # resets labels? no: keeps them
            e_slot = e.running_energy()
            before = e.replica_of_slot()
            start = step % 2 + 1
            want = D.swap_decisions(start, 1.0 / np.asarray(inp.tems), e_slot, step, seed)
            e.pt_swap(start, step, seed)
            after = e.replica_of_slot()
            expect = before.copy()
            for s in want:
                expect[s], expect[s + 1] = before[s + 1], before[s]
            assert np.array_equal(after, expect), (step, want)


@pytest.mark.parametrize("L,R", [(8, 6), (64, 80)])
def test_spin_transfers_agree_across_host_paths(L, R):
    """esp_set_spins / esp_get_spins through the pinned staging (in 256 MiB
    blocks of slots: the 64^3 x 80 case takes two) and, where the device
    reads and writes pageable host memory, directly: every mode leaves the
    same FP32 state (the FP64 input rounded) and returns it unchanged."""
    h = build_hamiltonian(sc_mcin(L, [(1e-3, NN)], list(np.linspace(5.0, 50.0, R))), check=False)
    rng = np.random.default_rng(L)
    v = rng.normal(size=(R, h.n, 3))
    s0 = v / np.linalg.norm(v, axis=2, keepdims=True)
    want = s0.astype(np.float32).astype(np.float64)
    with _engine(h, R) as e:
        _, direct = e.host_transfer()
        modes = [0, 1, 2, 3] if direct else [0]
        if not direct:
            with pytest.raises(RuntimeError):
                e.set_host_transfer(3)
        energies = []
        for m in modes:
            e.set_host_transfer(m)
            assert e.host_transfer() == (m, direct)
            e.set_spins(s0)
            energies.append(e.energy())
            out = e.get_spins()
            assert np.array_equal(out, want), m
            # into an array whose pages are already resident
            reused = np.full_like(out, 7.0)
            assert e.lib.esp_get_spins(e.h, reused.ctypes.data_as(ctypes.c_void_p)) == 0
            assert np.array_equal(reused, want), m
        for en in energies[1:]:
            assert np.array_equal(en, energies[0])
        e.set_host_transfer(-1)
        print(f"\nL={L} R={R}: direct host access {'supported' if direct else 'not supported'}, "
              f"default mode {e.host_transfer()[0]}")
