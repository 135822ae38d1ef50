"""Learned proposal on the GPU, through the C ABI.

* the sweep's fused BF16 forward pass and the training kernels' loss and
  gradient against the FP64 network of oracle/lp_oracle.c (same BF16-rounded
  weights and inputs; the GPU also rounds hidden activations and output
  gradients to BF16, so the bound is relative: 2e-2 on outputs, 5e-2 on the
  gradient norm);
* the collected training pairs against FP64 features of the oracle's local
  terms;
* the Metropolis-Hastings sampler with an untrained (far from optimal)
  network against the reference algorithm's chains within 3 sigma, so the
  proposal-density correction is exact;
* what training gains: lower loss, higher acceptance and a shorter
  integrated autocorrelation time of E than the plain sampler;
* the give-up path of the tcgen05 engine's bounded completion waits, made to
  run by the test hook esp_lp_force_tc_timeout (no real hang): esp_collect
  and esp_lp_forward return ESP_ETIMEOUT, the sweep makes no trial and
  writes no spin, and the handle works again after the hook is switched off.
"""
import numpy as np
import pytest

import oracle as O
from espins_gb300 import analysis
from espins_gb300.lib import ESP_ETIMEOUT, LP_NUM_PARAMS, Engine, EspError
from espins_gb300.tables import build_hamiltonian
from helpers import NN, NNN, energy_scale, exact_energy_axial, sc_mcin
from test_gpu_statistics import LEVELS, _check, _mean_sigma, _oracle_chains

pytestmark = pytest.mark.gpu

BLOCKS = [(0, 1536), (1536, 1664), (1664, 18048), (18048, 18176), (18176, 20736), (20736, 20756)]


def bf16(x):
    a = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)
    r = (a + np.uint32(0x7FFF) + ((a >> np.uint32(16)) & np.uint32(1))) & np.uint32(0xFFFF0000)
    return r.view(np.float32).astype(np.float64)


def _weights(seed, out_scale=0.1):
    rng = np.random.default_rng(seed)
    p = np.zeros(LP_NUM_PARAMS)
    p[0:1536] = rng.uniform(-1, 1, 1536) * np.sqrt(6 / 12)
    p[1536:1664] = rng.normal(size=128) * 0.1
    p[1664:18048] = rng.uniform(-1, 1, 16384) * np.sqrt(6 / 128)
    p[18048:18176] = rng.normal(size=128) * 0.1
    p[18176:20736] = rng.normal(size=2560) * out_scale
    p[20736:] = rng.normal(size=20) * out_scale
    return p.astype(np.float32)


def _rounded(p):
    """The parameters as the GPU sees them: BF16 weights, FP32 biases."""
    q = p.astype(np.float64)
    for lo, hi in (BLOCKS[0], BLOCKS[2], BLOCKS[4]):
        q[lo:hi] = bf16(p[lo:hi])
    return q


def _small_engine(R=2):
    inp = sc_mcin(4, [(1e-3, NN)], [10.0] * R)
    h = build_hamiltonian(inp)
    e = Engine(h.n, h.num_atoms, h.supercell, R)
    e.upload(h)
    e.set_temperatures(inp.tems)
    return e


def test_fused_forward_matches_fp64_network():
    p = _weights(1)
    rng = np.random.default_rng(2)
    x = rng.normal(size=(1000, 12)).astype(np.float32)   # ragged: not a multiple of 32
    with _small_engine() as e:
        e.lp_set_weights(p)
        assert np.array_equal(e.lp_weights(), p)
        got = e.lp_forward(x)
    want = O.lp_forward(_rounded(p), bf16(x))
    scale = np.abs(want).max()
    assert np.max(np.abs(got - want)) <= 2e-2 * scale, np.max(np.abs(got - want)) / scale


def test_tcgen05_forward_matches_fp64_network_and_mma_path():
    """The tcgen05 engine (128-row tiles, tensor-memory accumulators) against
    the FP64 network and the mma.sync engine on the same rows."""
    p = _weights(11)
    rng = np.random.default_rng(12)
    x = rng.normal(size=(1000, 12)).astype(np.float32)   # ragged: not a multiple of 128
    with _small_engine() as e:
        e.lp_set_weights(p)
        ref = e.lp_forward(x)
        e.lp_set_engine("tcgen05")
        got = e.lp_forward(x)
    want = O.lp_forward(_rounded(p), bf16(x))
    scale = np.abs(want).max()
    assert np.max(np.abs(got - want)) <= 2e-2 * scale, np.max(np.abs(got - want)) / scale
    # both engines round the hidden activations to bf16 the same way; only the
    # FP32 accumulation order differs
    assert np.max(np.abs(got - ref)) <= 5e-3 * scale, np.max(np.abs(got - ref)) / scale


def test_tcgen05_give_up_path_reports_timeout_and_writes_nothing():
    p = _weights(21)
    with _small_engine(R=4) as e:
        e.lp_set_weights(p)
        e.lp_set_engine("tcgen05")
        e.set_proposal("learned")
        e.init_spins("rand", seed=5)
        before, e_before = e.get_spins(), e.running_energy()
        e.lp_force_tc_timeout(True)
        e.begin(e.schedule(0, 2, 1, seed=9))
        e.advance(2)
        with pytest.raises(EspError) as ei:
            e.collect()
        assert ei.value.code == ESP_ETIMEOUT
        assert np.array_equal(e.get_spins(), before)
        assert np.array_equal(e.running_energy(), e_before)
        assert np.all(e.rejected()[:, 1] == 0)      # no trial was made, so none was rejected
        x = np.random.default_rng(3).normal(size=(200, 12)).astype(np.float32)
        with pytest.raises(EspError) as ei:
            e.lp_forward(x)
        assert ei.value.code == ESP_ETIMEOUT
        # hook off: a new run sweeps and collects normally
        e.lp_force_tc_timeout(False)
        e.begin(e.schedule(0, 2, 1, seed=9))
        e.advance(2)
        res = e.collect()
        assert not np.array_equal(e.get_spins(), before)
        assert res["rejected"][:, 1].sum() < 2 * 4 * e.n


@pytest.mark.parametrize("engine", ["mma", "tcgen05"])
@pytest.mark.parametrize("n", [1000, 4096])
def test_training_loss_and_gradient_match_fp64_network(engine, n):
    """Forward, loss head and backward GEMMs of a training step (mma.sync
    tiles, or tcgen05 with tensor-memory accumulators and the weight
    gradients split along the batch) against the FP64 network."""
    p = _weights(3)
    rng = np.random.default_rng(4)
    x = rng.normal(size=(n, 12)).astype(np.float32)
    s = rng.normal(size=(n, 3))
    s /= np.linalg.norm(s, axis=1, keepdims=True)
    t = np.column_stack([s, np.abs(rng.normal(size=n)) * 5]).astype(np.float32)
    with _small_engine() as e:
        e.lp_set_weights(p)
        e.lp_set_engine(engine)
        loss, g = e.lp_loss_grad(x, t)
        # deterministic: the same gradient again
        loss2, g2 = e.lp_loss_grad(x, t)
        assert loss2 == loss and np.array_equal(g2, g)
    lo, go = O.lp_loss_grad(_rounded(p), bf16(x), t.astype(np.float64))
    assert abs(loss - lo) <= 1e-2 * abs(lo), (loss, lo)
    assert np.linalg.norm(g - go) <= 5e-2 * np.linalg.norm(go)
    for a, b in BLOCKS:
        assert np.linalg.norm(g[a:b] - go[a:b]) <= 8e-2 * np.linalg.norm(go[a:b]) + 1e-7, (a, b)


def test_collected_pairs_match_oracle_features():
    inp = sc_mcin(6, [(1e-3, NN), (-6e-4, NNN)], [3.0, 9.0, 27.0], bq=5e-5, si=2e-4)
    h = build_hamiltonian(inp)
    R = len(inp.tems)
    rng = np.random.default_rng(5)
    v = rng.normal(size=(R, h.n, 3))
    spins = v / np.linalg.norm(v, axis=2, keepdims=True)
    H = O.Ham(h)
    with Engine(h.n, h.num_atoms, h.supercell, R) as e:
        e.upload(h)
        e.set_temperatures(inp.tems)
        e.set_spins(spins)
        colour, C = e.colouring()
        e.lp_reserve(h.n * R)
        c = 1
        n = e.lp_collect(c)
        sites = np.nonzero(colour == c)[0]
        assert n == len(sites) * R
        f_gpu, t_gpu = e.lp_data(0, n)
    ref_f, ref_t = [], []
    for r in range(R):
        sr = np.asarray(spins[r], dtype=np.float32).astype(np.float64)
        g, q = H.local_terms(sr.reshape(-1))
        for i in sites:
            ee, k0, f = O.lp_features(1.0 / inp.tems[r], 1.0, g[i], q[i], [0.0, 0.0, 1.0])
            ref_f.append(f)
            ref_t.append(np.concatenate([ee @ sr[i], [k0]]))
    ref_f, ref_t = np.array(ref_f), np.array(ref_t)
    key_r = np.column_stack([ref_t[:, 3], ref_t[:, :3]])
    key_g = np.column_stack([t_gpu[:, 3], t_gpu[:, :3]])
    for j in range(n):
        d = np.abs(key_r - key_g[j]).sum(axis=1)
        k = int(np.argmin(d))
        assert abs(t_gpu[j, 3] - ref_t[k, 3]) <= 1e-5 * (1 + ref_t[k, 3])
        assert np.max(np.abs(t_gpu[j, :3] - ref_t[k, :3])) <= 1e-4
        tol = 1e-2 * np.abs(ref_f[k]) + 2e-3
        assert np.all(np.abs(f_gpu[j] - ref_f[k]) <= tol), (f_gpu[j], ref_f[k])


COPIES = 4


def _learned_copies(h, tems, warm, mc, weights, seed=2468, engine="mma"):
    rt = np.repeat(np.asarray(tems, dtype=float), COPIES)
    with Engine(h.n, h.num_atoms, h.supercell, len(rt)) as e:
        e.upload(h)
        e.set_temperatures(rt)
        e.init_spins("ferro")
        e.lp_set_weights(weights)
        e.lp_set_engine(engine)
        e.set_proposal("learned")
        assert e.sweep_kernel()[0] == "learned"
        res = e.run(warm, mc, 1, pt=False, seed=seed, binning_level=LEVELS)
    d = res["data"].reshape(len(tems), COPIES, 6)
    b = res["binning"].reshape(len(tems), COPIES, len(LEVELS), 2)
    return [list(x) for x in d], [list(x) for x in b], res


def _independent_sites(tems):
    """Sites without couplings (J = 1e-12 eV): a Zeeman field along (1,1,0) and
    an easy-plane single-ion term along z, so every spin samples
    exp(-beta (f.s + Delta s_z^2)) on its own and <E>/N is a sphere integral."""
    extra = "ham_field = .true.\nbegin field_axes_cart\nFe 1 1 0 12.0\nend field_axes_cart\n"
    inp = sc_mcin(6, [(1e-12, NN)], tems, si=1.5e-4, extra=extra)
    return inp, build_hamiltonian(inp)


def _exact_energy_per_site(h, T):
    f = h.field_axis[0] * h.field_val[0]
    d = h.si_delta[0]
    ax = h.si_axis[0]
    nt, nph = 1200, 600
    ct = -1 + (np.arange(nt) + 0.5) * (2.0 / nt)
    ph = (np.arange(nph) + 0.5) * (2 * np.pi / nph)
    st = np.sqrt(1 - ct ** 2)
    s = np.stack([np.outer(st, np.cos(ph)), np.outer(st, np.sin(ph)), np.outer(ct, np.ones(nph))], -1).reshape(-1, 3)
    e = s @ f + d * (s @ ax) ** 2
    w = np.exp(-(e - e.min()) / T)
    return float((e * w).sum() / w.sum())


@pytest.mark.parametrize("engine", ["mma", "tcgen05"])
@pytest.mark.parametrize("out_scale", [0.0, 0.3])
def test_learned_sampler_is_exact_on_independent_sites(out_scale, engine):
    """Any network gives the exact single-site distribution: the zero network
    (the Heisenberg conditional, far from the true one because of the
    anisotropy) and a random one whose proposals point anywhere."""
    tems = [2.0, 6.0, 20.0]
    inp, h = _independent_sites(tems)
    warm, mc = 500, 20000
    gd, gb, res = _learned_copies(h, tems, warm, mc, _weights(8, out_scale=out_scale), engine=engine)
    for t, T in enumerate(tems):
        g, sg = _mean_sigma(gd[t], gb[t], h.n)
        want = _exact_energy_per_site(h, T)
        assert abs(g[0] - want) <= 3 * sg[0] + 1e-5 * abs(want), (T, g[0], want, sg[0])


def _offset_network(seed):
    """Weights whose outputs are a fixed offset from zero (W3 = 0, b3 set):
    each component's direction tilted by a few hundredths of a radian, its
    kappa changed by tens of per cent, unequal weights -- a proposal that
    differs from the target everywhere but still covers its peak."""
    p = _weights(seed, out_scale=0.0)
    b3 = np.zeros(20)
    for k in range(4):
        b3[5 * k] = 0.03 * (k - 1.5)
        b3[5 * k + 1] = 0.02 * (1.5 - k)
        b3[5 * k + 3] = 0.25 * (k - 1.5)
        b3[5 * k + 4] = 0.4 * k
    p[18176:20736] = 0.0
    p[20736:] = b3
    return p.astype(np.float32)


@pytest.mark.parametrize("engine", ["mma", "tcgen05"])
@pytest.mark.parametrize("net", ["zero", "offset"])
def test_learned_sampler_is_exact_at_large_kappa(net, engine):
    """The same exactness at the concentrations of a cold ordered lattice:
    independent sites in a 100 T field along z (67 K) with an easy-plane term
    along x, at 0.5-2 K, so the proposals' kappa is 30-130 -- where the
    sampler's inverse CDF and the log-densities of the Hastings ratio lose
    the most precision.  Two networks: the zero one (the Heisenberg
    conditional, which misses the anisotropy) and one with a fixed offset on
    every output.  (A random network's outputs point anywhere; at these
    concentrations a proposal that misses the target's peak by more than its
    width is almost never accepted, so such a chain stays near its start in
    any affordable run, which would say nothing about exactness.)"""
    tems = [0.5, 1.0, 2.0]
    extra = ("ham_field = .true.\nbegin field_axes_cart\nFe 0 0 1 100.0\nend field_axes_cart\n"
             "ham_singleion = .true.\nbegin singleion_axes_cart\nFe 1 0 0 2e-4\nend singleion_axes_cart\n")
    inp = sc_mcin(6, [(1e-12, NN)], tems, extra=extra)
    h = build_hamiltonian(inp)
    F = float(h.field_val[0] * h.field_axis[0][2])
    D = float(h.si_delta[0])
    warm, mc = 500, 20000
    w = _weights(9, out_scale=0.0) if net == "zero" else _offset_network(9)
    gd, gb, res = _learned_copies(h, tems, warm, mc, w, engine=engine)
    for t, T in enumerate(tems):
        g, sg = _mean_sigma(gd[t], gb[t], h.n)
        want = exact_energy_axial(F, D, T)
        print(f"\nT={T}: E/N {g[0]:.6f} +- {sg[0]:.6f}, exact {want:.6f}")
        assert abs(g[0] - want) <= 3 * sg[0] + 1e-6 * abs(want), (T, g[0], want, sg[0])


@pytest.mark.parametrize("engine", ["mma", "tcgen05"])
def test_learned_sampler_matches_reference_algorithm(engine):
    """An untrained network away from the prior on a frustrated lattice with
    biquadratic and single-ion terms: the exact Hastings ratio keeps the
    chain on the reference algorithm's stationary averages."""
    inp = sc_mcin(6, [(1e-3, NN), (-6e-4, NNN)], [4.0, 10.0, 25.0], bq=5e-5, si=2e-4)
    h = build_hamiltonian(inp)
    tems = inp.tems
    warm, mc = 2000, 30000
    gd, gb, res = _learned_copies(h, tems, warm, mc, _weights(7, out_scale=0.03), engine=engine)
    od, ob = _oracle_chains(h, tems, warm, mc, 515)
    _check(h, tems, gd, gb, od, ob, "learned MH")
    e = res["energy"]
    assert np.max(np.abs(e[:, 1] - e[:, 2])) <= 1e-5 * energy_scale(h)


def _acceptance(e, sweeps, n):
    rej = e.rejected()[:, 1]
    return 1.0 - rej / (sweeps * n)


def test_training_gains_over_plain_metropolis():
    inp = sc_mcin(8, [(1e-3, NN), (-6e-4, NNN)], [2.0, 5.0, 10.0], bq=5e-5, si=2e-4)
    h = build_hamiltonian(inp)
    tems = inp.tems
    R = len(tems)
    with Engine(h.n, h.num_atoms, h.supercell, R) as e:
        e.upload(h)
        e.set_temperatures(tems)
        e.init_spins("rand", seed=1)
        e.sweep(1000, 0, seed=4)
        colour, C = e.colouring()
        e.lp_reserve(200 * h.n * R)
        sweep = 1000
        for k in range(200):
            e.sweep(3, sweep, seed=4)
            sweep += 3
            e.lp_collect(k % C)
        e.lp_init(seed=9)
        loss = e.lp_train(600, batch=2048, lr=2e-3, seed=3)
        assert np.all(np.isfinite(loss))
        assert loss[-50:].mean() < loss[:10].mean() - 0.05, (loss[:10].mean(), loss[-50:].mean())

        # plain and learned chains from the same state: acceptance and tau_int(E)
        start = e.get_spins()
        out = {}
        for kind in ("plain", "learned"):
            e.set_spins(start)
            e.set_proposal(kind)
            e.set_series(20000)
            res = e.run(200, 20000, 1, pt=False, seed=77, binning_level=LEVELS)
            acc = 1.0 - res["rejected"][:, 1] / (20000 * h.n)
            ser = e.series()
            taus = np.array([analysis.tau_int(ser[:, t, 0]) for t in range(R)])
            out[kind] = (acc, taus)
    acc_p, tau_p = out["plain"]
    acc_l, tau_l = out["learned"]
    assert np.all(acc_l > acc_p + 0.1), (acc_p, acc_l)
    # the lowest temperature, where the plain sampler is slowest
    assert tau_l[0] < 0.7 * tau_p[0], (tau_p, tau_l)
