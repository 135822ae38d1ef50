"""The tiled sweep kernel (tiles of T cells + a one-cell halo of G replicas in
shared memory, 2x2x2 checkerboard of tiles).

It updates every site once per sweep with the random stream and arithmetic of
the other sweep kernels but in tile order, so it is checked by
* its stationary averages against the reference algorithm's chains (3 sigma),
* the running energy against a direct evaluation after many sweeps,
* independence of the trajectory from the grouping of replicas per CTA.
"""
import numpy as np
import pytest

from espins_gb300.lib import Engine
from espins_gb300.mcin import parse_mcin
from espins_gb300.tables import build_hamiltonian
from espins_gb300.workloads import BCC, BCC1, lattice_mcin
from helpers import N3, NN, NNN, energy_scale, sc_mcin
from test_gpu_statistics import COPIES, LEVELS, _check, _oracle_chains

pytestmark = pytest.mark.gpu


def _tile_copies(h, tems, warm, mc, geometry=None, seed=4321):
    rt = np.repeat(np.asarray(tems, dtype=float), COPIES)
    with Engine(h.n, h.num_atoms, h.supercell, len(rt)) as e:
        e.upload(h)
        e.set_temperatures(rt)
        e.set_sweep_kernel("tile")
        if geometry:
            e.set_tile_geometry(*geometry)
        assert e.sweep_kernel()[0] == "tile"
        e.init_spins("ferro")
        res = e.run(warm, mc, 1, pt=False, seed=seed, binning_level=LEVELS)
    d = res["data"].reshape(len(tems), COPIES, 6)
    b = res["binning"].reshape(len(tems), COPIES, len(LEVELS), 2)
    return [list(x) for x in d], [list(x) for x in b], res


def test_tiled_sweep_matches_reference_algorithm_sc_j123_dm_si():
    inp = sc_mcin(8, [(1e-3, NN), (3e-4, NNN), (-5e-5, N3)], [5.0, 12.0, 25.0], dm=1e-4, si=-3e-5)
    h = build_hamiltonian(inp)
    warm, mc = 2000, 30000
    gd, gb, res = _tile_copies(h, inp.tems, warm, mc, geometry=(2, 4))
    od, ob = _oracle_chains(h, inp.tems, warm, mc, 616)
    _check(h, inp.tems, gd, gb, od, ob, "tile sc")
    e = res["energy"]
    assert np.max(np.abs(e[:, 1] - e[:, 2])) <= 1e-5 * energy_scale(h)


def test_tiled_sweep_matches_reference_algorithm_bcc():
    inp = parse_mcin(lattice_mcin(BCC, 4, [(2e-3, BCC1), (5e-4, NN), (-1e-4, NNN)], tems=[15.0, 40.0, 80.0],
                                  single_ion=-5e-5), "bcc")
    h = build_hamiltonian(inp)
    warm, mc = 2000, 30000
    gd, gb, _ = _tile_copies(h, inp.tems, warm, mc, geometry=(2, 4))
    od, ob = _oracle_chains(h, inp.tems, warm, mc, 717)
    _check(h, inp.tems, gd, gb, od, ob, "tile bcc")


def test_tiled_trajectory_does_not_depend_on_replica_grouping():
    inp = sc_mcin(8, [(1e-3, NN), (-6e-4, NNN)], [2.0, 8.0, 30.0, 12.0], bq=5e-5, si=2e-4)
    h = build_hamiltonian(inp)
    rng = np.random.default_rng(4)
    v = rng.normal(size=(len(inp.tems), h.n, 3))
    s0 = v / np.linalg.norm(v, axis=2, keepdims=True)
    outs = []
    for T, G in [(2, 1), (2, 2), (2, 4), (4, 2)]:
        with Engine(h.n, h.num_atoms, h.supercell, len(inp.tems)) as e:
            e.upload(h)
            e.set_temperatures(inp.tems)
            e.set_sweep_kernel("tile")
            e.set_tile_geometry(T, G)
            assert e.tile_geometry() == (T, G, 0)
            e.set_spins(s0)
            e.sweep(30, 5, seed=9)
            outs.append(((T, G), e.get_spins(), e.rejected(), e.running_energy(), e.energy()))
    # the same tile size: identical trajectories whatever the grouping
    for g, s, rej, run, direct in outs[1:3]:
        assert np.array_equal(s, outs[0][1]), g
        assert np.array_equal(rej, outs[0][2]), g
    for g, s, rej, run, direct in outs:
        assert np.max(np.abs(run - direct)) <= 1e-5 * energy_scale(h), g
        assert np.allclose(np.linalg.norm(s, axis=2), 1.0, atol=2e-6)


@pytest.mark.parametrize("case", ["sc", "bcc"])
def test_pipelined_tiles_follow_the_one_tile_per_cta_kernel(case):
    """The persistent cp.async-pipelined variants (one CTA per SM with two box
    buffers, two CTAs per SM with one each) update the same tiles in the same
    order within each tile: identical trajectories."""
    tems = [3.0, 6.0, 12.0, 20.0, 30.0, 45.0, 60.0, 80.0]
    if case == "sc":
        inp = sc_mcin(16, [(1e-3, NN), (3e-4, NNN), (-5e-5, N3)], tems, dm=1e-4, si=-3e-5)
    else:
        inp = parse_mcin(lattice_mcin(BCC, 8, [(2e-3, BCC1), (5e-4, NN), (-1e-4, NNN)], tems=tems,
                                      single_ion=-5e-5), "bcc")
    h = build_hamiltonian(inp)
    rng = np.random.default_rng(12)
    v = rng.normal(size=(len(tems), h.n, 3))
    s0 = v / np.linalg.norm(v, axis=2, keepdims=True)
    outs = []
    for variant in (0, 1, 2):
        with Engine(h.n, h.num_atoms, h.supercell, len(tems)) as e:
            e.upload(h)
            e.set_temperatures(tems)
            e.set_sweep_kernel("tile")
            e.set_tile_geometry(4, 4, variant)
            assert e.tile_geometry() == (4, 4, variant)
            e.set_spins(s0)
            e.sweep(12, 3, seed=21)
            outs.append((e.get_spins(), e.rejected(), e.running_energy(), e.energy()))
    for k in (1, 2):
        assert np.array_equal(outs[0][0], outs[k][0])
        assert np.array_equal(outs[0][1], outs[k][1])
    for s, rej, run, direct in outs:
        assert np.max(np.abs(run - direct)) <= 1e-5 * energy_scale(h)
