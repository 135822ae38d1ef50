"""Many independent lattices: replica groups with exchange inside each group,
and batches of handles advanced by replayed CUDA graphs.

* k_pt_swap with groups takes the decisions of the host protocol applied to
  every group on its own;
* a batch advanced by graphs (several units per replay, plus a remainder
  advanced directly) ends in exactly the state of advancing every handle on
  its own: the kernels read their sweep / swap / measurement indices from
  device counters that each replay advances, so the random stream is the same;
* the autotuner reports a valid choice and the batch keeps running after it.
"""
import numpy as np
import pytest

from espins_gb300 import distributed as D
from espins_gb300.lib import Batch, Engine
from espins_gb300.tables import build_hamiltonian
from espins_gb300.workloads import batch_lattice_mcin
from helpers import NN, sc_mcin

pytestmark = pytest.mark.gpu


def test_pt_groups_take_the_host_protocol_decisions():
    G, ngroups = 5, 3
    tems = np.tile(np.geomspace(5.0, 40.0, G), ngroups)
    inp = sc_mcin(4, [(1e-3, NN)], list(np.geomspace(5.0, 40.0, G)))
    h = build_hamiltonian(inp)
    R = G * ngroups
    rng = np.random.default_rng(11)
    seed = 0xABCDEF0123
    with Engine(h.n, h.num_atoms, h.supercell, R) as e:
        e.upload(h)
        e.set_temperatures(tems)
        e.set_pt_groups(G)
        for step in range(8):
            v = rng.normal(size=(R, h.n, 3))
            e.set_spins(v / np.linalg.norm(v, axis=2, keepdims=True))
            e_slot = e.running_energy()
            before = e.replica_of_slot()
            start = step % 2 + 1
            want = D.swap_decisions(start, 1.0 / tems, e_slot, step, seed, group=G)
            e.pt_swap(start, step, seed)
            after = e.replica_of_slot()
            expect = before.copy()
            for s in want:
                assert s // G == (s + 1) // G     # never across lattices
                expect[s], expect[s + 1] = before[s + 1], before[s]
            assert np.array_equal(after, expect), (step, want)


def _handles(kinds):
    """One handle per (L, lattices, pt, kernel) in kinds, begun on its schedule
    ("tile:T,G,variant" fixes the tiled kernel's geometry)."""
    out = []
    for L, nlat, pt, kernel in kinds:
        inp = batch_lattice_mcin(L, replicas=4)
        h = build_hamiltonian(inp, check=False)
        R = 4 * nlat
        e = Engine(h.n, h.num_atoms, h.supercell, R)
        e.upload(h)
        e.set_temperatures(np.tile(inp.tems, nlat))
        e.set_pt_groups(4)
        if kernel.startswith("tile:"):
            e.set_tile_geometry(*(int(x) for x in kernel[5:].split(",")))
            kernel = "tile"
        e.set_sweep_kernel(kernel)
        e.init_spins("rand", seed=L)
        e.set_series(64)
        s = e.schedule(20, 500, 1, pt=pt, pt_steps_swap=3 if pt else 1, seed=900 + L, binning_level=[1, 2, 3])
        e.begin(s)
        out.append(e)
    return out


KINDS = [(4, 2, True, "ell"), (8, 3, True, "cluster"), (6, 1, False, "ell"), (12, 2, False, "cluster"),
         (16, 2, True, "tile:4,8,2")]


def test_batch_graph_replays_equal_separate_advances():
    n_units = 11
    ref = _handles(KINDS)
    for e in ref:
        e.advance(n_units)
    want = [(e.collect(), e.get_spins(), e.series()) for e in ref]
    got_h = _handles(KINDS)
    with Batch(got_h) as b:
        b.set_units_per_graph(4)          # two replays of 4 units, then 3 units directly
        b.advance(n_units)
    for e, (rw, sw, serw) in zip(got_h, want):
        rg = e.collect()
        assert np.array_equal(e.get_spins(), sw)
        for k in ("rejected", "data", "binning", "num_swaps", "map", "energy", "pm"):
            assert np.array_equal(rg[k], rw[k]), k
        assert np.array_equal(e.series(), serw)
    for e in ref + got_h:
        e.close()


def test_autotuner_chooses_and_batch_keeps_running():
    hs = _handles(KINDS)
    l0 = [e.launch_count() for e in hs]
    with Batch(hs) as b:
        t = b.tune(units=2)
        assert t["units_per_graph"] in (1, 2, 4, 8)
        assert t["us_per_unit"] > 0
        for i, (L, _, _, _) in enumerate(KINDS):
            assert t["ell_us"][i] > 0
            if t["cluster_us"][i] > 0:
                assert (t["kernel"][i] != "ell") == (t["cluster_us"][i] < t["ell_us"][i])
            else:
                assert t["kernel"][i] == "ell"
        b.advance(5)
    for e, l in zip(hs, l0):
        r = e.collect()
        assert np.all(np.isfinite(r["data"]))
        assert e.launch_count() > l
        # the running energy still equals a direct evaluation
        assert np.allclose(r["energy"][:, 1], r["energy"][:, 2], rtol=1e-5, atol=1e-3)
        e.close()
