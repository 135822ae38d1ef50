"""The allocation-free direct energy, esp_energy_noalloc.

It exists for hosts that cannot let a library call cudaMalloc: the caller owns
every device buffer (here torch allocates them, standing in for such a host)
and the entry point's partial sums live in a fixed array inside the library.
Its results must match the regular entry point esp_energy, which allocates its
scratch per handle, and the FP64 oracle's energy_get of the same (FP32-rounded)
spins, within the energy tolerance of the parity tests, on two calls in a row
with different inputs; the second Hamiltonian adds a Zeeman field, so every
term of energy_get (exchange, biquadratic, DM, single-ion, field) is covered.
The file sorts last so that a stop-at-first-failure run has run every other
test before it.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from espins_gb300 import lib as L
from espins_gb300.tables import build_hamiltonian
from helpers import ENERGY_RTOL, NN, NNN, energy_scale, sc_mcin

pytestmark = pytest.mark.gpu


def _device_args(torch, h, spins):
    """Device copies of the reference-layout tables and spins (owned by torch)."""
    dev = torch.device("cuda")
    keep = []

    def d(a, dt):
        t = torch.as_tensor(np.ascontiguousarray(a), device=dev).to(dt).contiguous()
        keep.append(t)
        return t.data_ptr()

    a = L.EnergyArgs()
    a.num_sites, a.num_atoms, a.num_replicas = h.n, h.num_atoms, spins.shape[0]
    a.spins = d(spins, torch.float64)                       # (R, N, 3) == spin_matrix(3,N,R)
    a.j_nn, a.j_nbors, a.j_val = d(h.jij.nn, torch.int32), d(h.jij.nb + 1, torch.int32), d(h.jij.val, torch.float64)
    if h.bij is not None:
        a.b_nn, a.b_nbors, a.b_val = d(h.bij.nn, torch.int32), d(h.bij.nb + 1, torch.int32), d(h.bij.val, torch.float64)
    if h.dij is not None:
        a.d_nn, a.d_nbors, a.d_val = d(h.dij.nn, torch.int32), d(h.dij.nb + 1, torch.int32), d(h.dij.val, torch.float64)
    if h.si_axis is not None:
        a.si_axis, a.si_delta = d(h.si_axis, torch.float64), d(h.si_delta, torch.float64)
    if h.field_axis is not None:
        a.field_axis, a.field_val = d(h.field_axis, torch.float64), d(h.field_val, torch.float64)
    return a, keep


def _regular_energy(h, spins, tems):
    with L.Engine(h.n, h.num_atoms, h.supercell, spins.shape[0]) as e:
        e.upload(h)
        e.set_temperatures(tems)
        e.set_spins(spins)
        return e.energy()


def test_energy_noalloc_matches_esp_energy_twice():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    lib = L.load()
    field = "ham_field = .true.\nbegin field_axes_cart\nFe 0.3 -0.2 0.9 2.5\nend field_axes_cart\n"
    rng = np.random.default_rng(11)
    stream = torch.cuda.current_stream()
    for call, (R, extra) in enumerate(((3, ""), (5, field))):
        inp = sc_mcin(6, [(1e-3, NN), (3e-4, NNN)], [5.0, 12.0, 25.0], bq=1e-4, dm=2e-4, si=-3e-5, extra=extra)
        h = build_hamiltonian(inp)
        assert (h.field_axis is not None) == bool(extra)
        tol = ENERGY_RTOL * energy_scale(h)
        v = rng.normal(size=(R, h.n, 3))
        spins = v / np.linalg.norm(v, axis=2, keepdims=True)
        ref = _regular_energy(h, spins, np.linspace(5.0, 25.0, R))
        H = O.Ham(h)
        oracle = np.array([H.energy(np.float32(s).astype(np.float64).reshape(-1)) for s in spins])
        args, keep = _device_args(torch, h, spins)
        out = torch.full((R,), float("nan"), dtype=torch.float64, device="cuda")
        rc = lib.esp_energy_noalloc(C.byref(args), C.c_void_p(out.data_ptr()), C.c_void_p(stream.cuda_stream))
        assert rc == L.ESP_OK, L.last_global_error()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.max(np.abs(got - ref)) <= tol, (call, got, ref, tol)
        assert np.max(np.abs(got - oracle)) <= tol, (call, got, oracle, tol)


def test_energy_noalloc_rejects_too_many_replicas():
    torch = pytest.importorskip("torch")
    lib = L.load()
    inp = sc_mcin(4, [(1e-3, NN)], [5.0])
    h = build_hamiltonian(inp)
    spins = np.zeros((1, h.n, 3)); spins[..., 2] = 1.0
    args, keep = _device_args(torch, h, spins)
    args.num_replicas = 4097
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = lib.esp_energy_noalloc(C.byref(args), C.c_void_p(out.data_ptr()), None)
    assert rc == L.ESP_EINVAL
    assert "4096" in L.last_global_error()
