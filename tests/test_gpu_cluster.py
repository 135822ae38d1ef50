"""The cluster-resident sweep kernel against the ELL kernel.

Both kernels use the same colouring, the same Philox counter (site, replica,
sweep) and the same order of the local-field sums, so from the same state they
must produce the same trajectory; whole plain and parallel-tempering runs must
give the same accumulators and counters.  Spins may differ only by FP32
contraction differences (<= 1e-5), which must not change any decision.
"""
import numpy as np
import pytest

from espins_gb300.lib import Engine
from espins_gb300.tables import build_hamiltonian
from espins_gb300.workloads import BCC, BCC1, NN, NNN, N3, lattice_mcin
from espins_gb300.mcin import parse_mcin
from helpers import energy_scale, sc_mcin

pytestmark = pytest.mark.gpu


def _cases():
    return {
        "sc_j1": sc_mcin(8, [(1e-3, NN)], [3.0, 10.0, 30.0]),
        "sc_j123_dm_si": sc_mcin(8, [(1e-3, NN), (3e-4, NNN), (-5e-5, N3)], [5.0, 20.0, 40.0], dm=1e-4, si=-3e-5),
        "sc_j1j2_bq_si": sc_mcin(12, [(1e-3, NN), (-6e-4, NNN)], [2.0, 8.0, 30.0, 12.0], bq=5e-5, si=2e-4),
        # 4096 sites: one CTA per replica stages its slab through the
        # contiguous buffer, two or more gather it directly
        "sc16_j1j2_dm": sc_mcin(16, [(1e-3, NN), (3e-4, NNN)], [3.0, 12.0, 40.0], dm=1e-4),
        # 32768 sites: slabs of 12 + 10 + 10 planes on 3 CTAs, staged
        "sc32_j1_dm": sc_mcin(32, [(1e-3, NN)], [4.0, 20.0], dm=2e-4),
        "bcc_pt": parse_mcin(lattice_mcin(BCC, 8, [(2e-3, BCC1), (5e-4, NN), (-1e-4, NNN)], tems=[10.0, 20.0, 40.0, 80.0],
                                          single_ion=-5e-5, pt=True, pt_steps_swap=5), "bcc"),
    }


def _engine(h, tems, kind):
    e = Engine(h.n, h.num_atoms, h.supercell, len(tems))
    e.upload(h)
    e.set_temperatures(tems)
    e.set_sweep_kernel(kind)
    return e


@pytest.mark.parametrize("case", ["sc_j1", "sc_j123_dm_si", "sc_j1j2_bq_si", "bcc_pt"])
@pytest.mark.parametrize("mode", [0, 1])
def test_cluster_kernel_follows_the_ell_trajectory(case, mode):
    inp = _cases()[case]
    h = build_hamiltonian(inp)
    rng = np.random.default_rng(5)
    v = rng.normal(size=(len(inp.tems), h.n, 3))
    s0 = v / np.linalg.norm(v, axis=2, keepdims=True)
    out = {}
    for kind in ("ell", "cluster"):
        with _engine(h, inp.tems, kind) as e:
            assert e.sweep_kernel()[0] == kind
            e.set_spins(s0)
            e.sweep(25, 3, seed=77, mode=mode, tilt=0.4)
            out[kind] = (e.get_spins(), e.running_energy(), e.rejected())
    a, b = out["ell"], out["cluster"]
    assert np.max(np.abs(a[0] - b[0])) <= 1e-5
    assert np.array_equal(a[2], b[2])
    assert np.max(np.abs(a[1] - b[1])) <= 1e-6 * h.n * 40.0


@pytest.mark.parametrize("case,pt", [("sc_j1j2_bq_si", False), ("bcc_pt", True)])
def test_cluster_kernel_runs_match_ell_runs(case, pt):
    inp = _cases()[case]
    h = build_hamiltonian(inp)
    res = {}
    for kind in ("ell", "cluster"):
        with _engine(h, inp.tems, kind) as e:
            e.init_spins("ferro")
            res[kind] = e.run(40, 300, 2, pt=pt, pt_steps_swap=5, seed=31, binning_level=[1, 2, 3, 4])
    a, b = res["ell"], res["cluster"]
    assert np.array_equal(a["rejected"], b["rejected"])
    assert np.array_equal(a["num_swaps"], b["num_swaps"])
    assert np.array_equal(a["map"], b["map"])
    # the same decisions (above, exactly); the accumulators differ only by the
    # order in which the kernels add their FP32 per-sweep sums into the FP64
    # running energy and magnetisation (a few parts in 1e7 of the small net
    # magnetisation's moments)
    assert np.allclose(a["data"], b["data"], rtol=1e-6, atol=1e-9)
    assert np.allclose(a["pm"], b["pm"], rtol=0, atol=1e-9)
    assert np.allclose(a["binning"], b["binning"], rtol=1e-5, atol=1e-12)
    # running energies: the kernels add their FP32 per-sweep sums in different
    # orders; the direct energies (column 2) agree to FP64 summation order
    assert np.max(np.abs(a["energy"][:, :2] - b["energy"][:, :2])) <= 1e-5 * energy_scale(h)
    assert np.allclose(a["energy"][:, 2], b["energy"][:, 2], rtol=1e-12, atol=1e-9)


def test_cluster_kernel_is_chosen_for_invariant_lattices_only():
    inp = sc_mcin(8, [(1e-3, NN)], [5.0, 6.0])
    h = build_hamiltonian(inp)
    with Engine(h.n, h.num_atoms, h.supercell, 2) as e:
        e.upload(h)
        e.set_temperatures([5.0, 6.0])
        assert e.sweep_kernel()[0] == "cluster"
    inp.boundary_open = True
    h = build_hamiltonian(inp)
    with Engine(h.n, h.num_atoms, h.supercell, 2, open_boundary=True) as e:
        e.upload(h)
        e.set_temperatures([5.0, 6.0])
        assert e.sweep_kernel()[0] == "ell"


@pytest.mark.parametrize("case", ["sc_j1j2_bq_si", "bcc_pt", "sc16_j1j2_dm", "sc32_j1_dm"])
def test_trajectory_does_not_depend_on_cluster_geometry(case):
    """Every (CTAs per replica, threads per CTA) geometry the GPU can run gives
    the same spins and rejected counts (same colour order and random stream);
    only the FP32 grouping of the per-sweep sums may differ.  CTA counts that
    do not divide the z plane pairs give slabs of two heights (e.g. 4 + 4 + 2
    + 2 planes of a 12-plane lattice on 4 CTAs)."""
    inp = _cases()[case]
    h = build_hamiltonian(inp)
    rng = np.random.default_rng(8)
    v = rng.normal(size=(len(inp.tems), h.n, 3))
    s0 = v / np.linalg.norm(v, axis=2, keepdims=True)
    outs = []
    geoms = [(cs, nt, sp) for cs in (1, 2, 3, 4, 5) for nt, sp in ((512, 1), (512, 2), (256, 1))]
    for cs, nt, sp in geoms:
        with _engine(h, inp.tems, "cluster") as e:
            try:
                e.set_cluster_geometry(cs, nt, sp)
            except Exception:
                continue          # not possible for this lattice / GPU
            assert e.cluster_geometry() == (cs, nt, sp)
            e.set_spins(s0)
            e.sweep(20, 11, seed=5)
            outs.append(((cs, nt), e.get_spins(), e.rejected(), e.running_energy()))
    assert len(outs) >= 2, [o[0] for o in outs]
    pairs = h.supercell[2] // 2
    assert any(pairs % g[0] for g, *_ in outs), [o[0] for o in outs]   # an uneven split ran
    for g, s, rej, en in outs[1:]:
        assert np.array_equal(s, outs[0][1]), g
        assert np.array_equal(rej, outs[0][2]), g
        assert np.max(np.abs(en - outs[0][3])) <= 1e-6 * h.n * 40.0, g


def test_a_smaller_lattice_set_up_later_does_not_break_a_larger_ones_launches():
    """The dynamic shared-memory limit belongs to the kernel function, not to
    a handle: configuring the cluster path of a small lattice after a large
    one (same kernel, less shared memory) must leave the large one's
    launches valid."""
    big = sc_mcin(16, [(1e-3, NN)], [3.0, 10.0])
    small = sc_mcin(8, [(1e-3, NN)], [3.0, 10.0])
    hb, hs = build_hamiltonian(big), build_hamiltonian(small)
    with _engine(hb, big.tems, "cluster") as eb:
        eb.set_cluster_geometry(1, 512, 1)
        eb.init_spins("ferro")
        with _engine(hs, small.tems, "cluster") as es:
            es.set_cluster_geometry(1, 512, 1)
            es.init_spins("ferro")
            es.sweep(2, 1, seed=3)
        eb.sweep(2, 1, seed=3)
        assert eb.sweep_kernel()[0] == "cluster"
        assert np.all(np.isfinite(eb.running_energy()))


def test_spin_copies_stay_consistent_across_kernels_and_reads():
    """The cluster path leaves the state in its slab copy and brings the spin
    arrays back only when something reads them; the arrays' writers make the
    slab stale.  Reading the spins in the middle of a run changes nothing
    (same final spins and counters as a run without the read), and switching
    between the cluster, ELL and cluster kernels again keeps the running
    energy equal to the direct one."""
    inp = _cases()["sc16_j1j2_dm"]   # 4096 sites: one CTA per replica, staged slab
    h = build_hamiltonian(inp)
    rng = np.random.default_rng(8)
    v = rng.normal(size=(len(inp.tems), h.n, 3))
    s0 = v / np.linalg.norm(v, axis=2, keepdims=True)
    out = []
    for read in (False, True):
        with _engine(h, inp.tems, "cluster") as e:
            e.set_cluster_geometry(1, 512, 1)
            e.set_spins(s0)
            e.sweep(6, 0, seed=3)
            if read:
                mid = e.get_spins()
                assert np.all(np.isfinite(mid)) and not np.array_equal(mid, s0)
            e.sweep(6, 6, seed=3)
            out.append((e.get_spins(), e.rejected(), e.running_energy()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    with _engine(h, inp.tems, "cluster") as e:
        e.set_cluster_geometry(1, 512, 1)
        e.set_spins(s0)
        tol = 1e-5 * energy_scale(h)
        for k, kind in enumerate(("cluster", "ell", "cluster", "ell")):
            e.set_sweep_kernel(kind)
            e.sweep(4, 4 * k, seed=9)
            run, direct = e.running_energy(), e.energy()
            assert np.max(np.abs(run - direct)) <= tol, (kind, run - direct)
