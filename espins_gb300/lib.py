"""ctypes binding of libespins_gpu.so (the C ABI in include/espins_gpu.h).

This is the same binding a Python host of the library would write; a Fortran
host binds the same entry points with an iso_c_binding interface block.  There
is no CPU fallback: if the library cannot be loaded or no GPU is present, the
calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from . import build as _build

ESP_OK, ESP_EINVAL, ESP_ECUDA, ESP_ENOMEM, ESP_ESTATE, ESP_ETIMEOUT, ESP_ECOLOR = range(7)

EXPORTED = [
    "esp_create", "esp_destroy", "esp_last_error", "esp_set_stream", "esp_upload_tables",
    "esp_set_temperatures", "esp_set_spins", "esp_init_spins", "esp_run", "esp_begin",
    "esp_advance", "esp_collect", "esp_sweep",
    "esp_sweep_colour", "esp_pt_swap", "esp_energy", "esp_running_energy",
    "esp_running_magnetization", "esp_local_terms", "esp_get_spins", "esp_get_colouring",
    "esp_get_rejected", "esp_get_replica_of_slot", "esp_num_freq", "esp_launch_count",
    "esp_energy_noalloc", "esp_set_sweep_kernel", "esp_get_sweep_kernel", "esp_set_series", "esp_get_series",
    "esp_lp_num_params", "esp_lp_init_weights", "esp_lp_set_weights", "esp_lp_get_weights", "esp_lp_reserve",
    "esp_lp_collect", "esp_lp_get_data", "esp_lp_train", "esp_lp_loss_grad", "esp_lp_forward", "esp_lp_set_engine",
    "esp_lp_force_tc_timeout",
    "esp_set_proposal", "esp_get_proposal",
    "esp_set_pt_groups", "esp_set_cluster_geometry", "esp_get_cluster_geometry",
    "esp_set_tile_geometry", "esp_get_tile_geometry", "esp_batch_create", "esp_batch_destroy", "esp_batch_last_error",
    "esp_batch_set_units_per_graph", "esp_batch_advance", "esp_batch_tune",
    "esp_set_observables", "esp_collect_observables", "esp_set_spin_correlation", "esp_collect_spin_correlation",
    "esp_set_structure_factor", "esp_collect_structure_factor", "esp_set_host_transfer", "esp_get_host_transfer",
]

OBS_ORDER_PARAMETER, OBS_STAGGERED = 1, 2

LP_NUM_PARAMS = 20756
LP_IN, LP_OUT = 12, 20


class EspError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"libespins_gpu error {code}: {msg}")
        self.code = code


class LpTrainOpts(C.Structure):
    _fields_ = [("steps", C.c_int32), ("batch", C.c_int32), ("lr", C.c_double), ("beta1", C.c_double),
                ("beta2", C.c_double), ("eps", C.c_double), ("seed", C.c_uint64)]


class BatchTuning(C.Structure):
    _fields_ = [("units_per_graph", C.c_int32), ("us_per_unit", C.c_double), ("kernel", C.c_void_p),
                ("ell_us", C.c_void_p), ("cluster_us", C.c_void_p), ("graph_us", C.c_void_p),
                ("cluster_size", C.c_void_p), ("cluster_threads", C.c_void_p), ("cluster_sites", C.c_void_p)]


class Dims(C.Structure):
    _fields_ = [("num_sites", C.c_int32), ("num_atoms", C.c_int32), ("supercell", C.c_int32 * 3),
                ("num_replicas", C.c_int32), ("open_boundary", C.c_int32)]


class Tables(C.Structure):
    _fields_ = [("mag", C.c_void_p),
                ("j_maxnb", C.c_int32), ("j_nn", C.c_void_p), ("j_nbors", C.c_void_p), ("j_val", C.c_void_p),
                ("b_maxnb", C.c_int32), ("b_nn", C.c_void_p), ("b_nbors", C.c_void_p), ("b_val", C.c_void_p),
                ("d_maxnb", C.c_int32), ("d_nn", C.c_void_p), ("d_nbors", C.c_void_p), ("d_val", C.c_void_p),
                ("si_axis", C.c_void_p), ("si_delta", C.c_void_p),
                ("field_axis", C.c_void_p), ("field_val", C.c_void_p)]


class Schedule(C.Structure):
    _fields_ = [("steps_warmup", C.c_int64), ("steps_mc", C.c_int64), ("steps_measure", C.c_int64),
                ("pt", C.c_int32), ("mcarlo_mode", C.c_int32), ("pt_steps_swap", C.c_int64),
                ("tilt_angles_max", C.c_double), ("seed", C.c_uint64), ("lbinerror", C.c_int32),
                ("num_binning_level", C.c_int32), ("binning_level", C.c_void_p)]


class Results(C.Structure):
    _fields_ = [("rejected", C.c_void_p), ("steps_tot", C.c_void_p), ("energy", C.c_void_p),
                ("data", C.c_void_p), ("pm", C.c_void_p), ("binning", C.c_void_p),
                ("num_swaps", C.c_void_p), ("map", C.c_void_p), ("steps_mc_eff", C.c_int64)]


class ObsResults(C.Structure):
    _fields_ = [("data", C.c_void_p), ("pm_op", C.c_void_p), ("pm_sm", C.c_void_p), ("binning", C.c_void_p)]


class EnergyArgs(C.Structure):
    """esp_energy_args: device pointers in the reference's layouts."""
    _fields_ = [("num_sites", C.c_int32), ("num_atoms", C.c_int32), ("num_replicas", C.c_int32),
                ("spins", C.c_void_p),
                ("j_nn", C.c_void_p), ("j_nbors", C.c_void_p), ("j_val", C.c_void_p),
                ("b_nn", C.c_void_p), ("b_nbors", C.c_void_p), ("b_val", C.c_void_p),
                ("d_nn", C.c_void_p), ("d_nbors", C.c_void_p), ("d_val", C.c_void_p),
                ("si_axis", C.c_void_p), ("si_delta", C.c_void_p),
                ("field_axis", C.c_void_p), ("field_val", C.c_void_p)]


class SweepOpts(C.Structure):
    _fields_ = [("mcarlo_mode", C.c_int32), ("tilt_angles_max", C.c_double), ("seed", C.c_uint64),
                ("phase", C.c_int32)]


_lib = None


def load(build_if_missing: bool = True):
    """Load libespins_gpu.so from the package directory (building it if asked)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise OSError(f"{path} is missing: run espins_gb300.build.build()")
        _build.build()
    lib = C.CDLL(path)
    P, vp = C.POINTER, C.c_void_p
    lib.esp_create.argtypes = [P(Dims), P(vp)]
    lib.esp_destroy.argtypes = [vp]
    lib.esp_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
    lib.esp_set_stream.argtypes = [vp, vp]
    lib.esp_upload_tables.argtypes = [vp, P(Tables)]
    lib.esp_set_temperatures.argtypes = [vp, vp]
    lib.esp_set_spins.argtypes = [vp, vp]
    lib.esp_init_spins.argtypes = [vp, C.c_int32, C.c_uint64]
    lib.esp_run.argtypes = [vp, P(Schedule), P(Results)]
    lib.esp_begin.argtypes = [vp, P(Schedule)]
    lib.esp_advance.argtypes = [vp, C.c_int64]
    lib.esp_collect.argtypes = [vp, P(Results)]
    lib.esp_sweep.argtypes = [vp, C.c_int64, C.c_int64, P(SweepOpts)]
    lib.esp_sweep_colour.argtypes = [vp, C.c_int32, C.c_int64, P(SweepOpts)]
    lib.esp_pt_swap.argtypes = [vp, C.c_int32, C.c_int64, C.c_uint64]
    for f in ("esp_energy", "esp_running_energy", "esp_running_magnetization", "esp_get_spins",
              "esp_get_rejected", "esp_get_replica_of_slot"):
        getattr(lib, f).argtypes = [vp, vp]
    lib.esp_local_terms.argtypes = [vp, vp, vp]
    lib.esp_get_colouring.argtypes = [vp, vp, P(C.c_int32)]
    lib.esp_num_freq.argtypes = [vp, P(C.c_int32)]
    lib.esp_launch_count.argtypes = [vp, P(C.c_int64)]
    lib.esp_energy_noalloc.argtypes = [P(EnergyArgs), vp, vp]
    lib.esp_set_sweep_kernel.argtypes = [vp, C.c_int32]
    lib.esp_set_series.argtypes = [vp, C.c_int64]
    lib.esp_get_series.argtypes = [vp, vp, P(C.c_int64)]
    lib.esp_get_sweep_kernel.argtypes = [vp, P(C.c_int32), P(C.c_int32)]
    lib.esp_lp_num_params.argtypes = []
    lib.esp_lp_init_weights.argtypes = [vp, C.c_uint64]
    lib.esp_lp_set_weights.argtypes = [vp, vp]
    lib.esp_lp_get_weights.argtypes = [vp, vp]
    lib.esp_lp_reserve.argtypes = [vp, C.c_int64]
    lib.esp_lp_collect.argtypes = [vp, C.c_int32, P(C.c_int64)]
    lib.esp_lp_get_data.argtypes = [vp, C.c_int64, C.c_int64, vp, vp]
    lib.esp_lp_train.argtypes = [vp, P(LpTrainOpts), vp]
    lib.esp_lp_loss_grad.argtypes = [vp, vp, vp, C.c_int64, P(C.c_double), vp]
    lib.esp_lp_forward.argtypes = [vp, vp, C.c_int64, vp]
    lib.esp_lp_set_engine.argtypes = [vp, C.c_int32]
    lib.esp_lp_force_tc_timeout.argtypes = [vp, C.c_int32]
    lib.esp_set_proposal.argtypes = [vp, C.c_int32]
    lib.esp_get_proposal.argtypes = [vp, P(C.c_int32)]
    lib.esp_set_pt_groups.argtypes = [vp, C.c_int32]
    lib.esp_set_cluster_geometry.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32]
    lib.esp_set_tile_geometry.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32]
    lib.esp_get_tile_geometry.argtypes = [vp, P(C.c_int32), P(C.c_int32), P(C.c_int32)]
    lib.esp_set_host_transfer.argtypes = [vp, C.c_int32]
    lib.esp_get_host_transfer.argtypes = [vp, P(C.c_int32), P(C.c_int32)]
    lib.esp_get_cluster_geometry.argtypes = [vp, P(C.c_int32), P(C.c_int32), P(C.c_int32)]
    lib.esp_batch_create.argtypes = [vp, C.c_int32, vp, P(vp)]
    lib.esp_batch_destroy.argtypes = [vp]
    lib.esp_batch_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
    lib.esp_batch_set_units_per_graph.argtypes = [vp, C.c_int32]
    lib.esp_batch_advance.argtypes = [vp, C.c_int64]
    lib.esp_batch_tune.argtypes = [vp, C.c_int32, P(BatchTuning)]
    for f in EXPORTED:
        getattr(lib, f).restype = C.c_int
    _lib = lib
    return lib


def last_global_error() -> str:
    """esp_last_error(NULL, ...): the message of a failed call without a handle."""
    buf = C.create_string_buffer(512)
    load().esp_last_error(None, buf, 512)
    return buf.value.decode()


def _p(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


class Engine:
    """One lattice with R replicas on the GPU (an ``esp_handle``)."""

    def __init__(self, n: int, num_atoms: int, supercell, num_replicas: int, open_boundary: bool = False):
        self.lib = load()
        d = Dims()
        d.num_sites, d.num_atoms = int(n), int(num_atoms)
        for c in range(3):
            d.supercell[c] = int(supercell[c])
        d.num_replicas, d.open_boundary = int(num_replicas), int(bool(open_boundary))
        h = C.c_void_p()
        rc = self.lib.esp_create(C.byref(d), C.byref(h))
        if rc != ESP_OK:
            buf = C.create_string_buffer(512)
            self.lib.esp_last_error(None, buf, 512)
            raise EspError(rc, buf.value.decode())
        self.h = h
        self.n, self.na, self.R = int(n), int(num_atoms), int(num_replicas)
        self._keep = []

    # -- plumbing -------------------------------------------------------------
    def _check(self, rc: int):
        if rc != ESP_OK:
            buf = C.create_string_buffer(1024)
            self.lib.esp_last_error(self.h, buf, 1024)
            raise EspError(rc, buf.value.decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.esp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- data in --------------------------------------------------------------
    def upload(self, ham) -> None:
        """Upload a Hamiltonian (espins_gb300.tables.Hamiltonian or equivalent)."""
        keep = []

        def arr(a, dt):
            a = np.ascontiguousarray(a, dtype=dt)
            keep.append(a)
            return a.ctypes.data

        t = Tables()
        t.mag = arr(ham.mag, np.float64)

        def ell(tab):
            nn = arr(tab.nn, np.int32)
            nb1 = (np.asarray(tab.nb, dtype=np.int32) + 1)
            nbp = arr(nb1, np.int32)
            # (maxnb, N[, 3]) C order is the memory order of jij_matrix(N,maxnb)
            # and dij_matrix(3,N,maxnb)
            val = arr(tab.val, np.float64)
            return int(tab.nb.shape[0]), nn, nbp, val

        t.j_maxnb, t.j_nn, t.j_nbors, t.j_val = ell(ham.jij)
        if getattr(ham, "bij", None) is not None:
            t.b_maxnb, t.b_nn, t.b_nbors, t.b_val = ell(ham.bij)
        if getattr(ham, "dij", None) is not None:
            t.d_maxnb, t.d_nn, t.d_nbors, t.d_val = ell(ham.dij)
        if getattr(ham, "si_axis", None) is not None:
            t.si_axis = arr(ham.si_axis, np.float64)
            t.si_delta = arr(ham.si_delta, np.float64)
        if getattr(ham, "field_axis", None) is not None:
            t.field_axis = arr(ham.field_axis, np.float64)
            t.field_val = arr(ham.field_val, np.float64)
        self._check(self.lib.esp_upload_tables(self.h, C.byref(t)))
        self._obs = 0   # new tables clear the optional measurements
        self._sc = None
        self._sf = 0

    def set_temperatures(self, tems) -> None:
        t = np.ascontiguousarray(tems, dtype=np.float64)
        assert t.size == self.R
        self._check(self.lib.esp_set_temperatures(self.h, _p(t)))

    def set_spins(self, spins: np.ndarray) -> None:
        """spins: (R, N, 3) in temperature-slot order."""
        s = np.ascontiguousarray(spins, dtype=np.float64)
        assert s.shape == (self.R, self.n, 3)
        self._check(self.lib.esp_set_spins(self.h, _p(s)))

    def init_spins(self, kind: str = "ferro", seed: int = 0) -> None:
        k = {"ferro": 0, "rand": 1}[kind]
        self._check(self.lib.esp_init_spins(self.h, k, int(seed) & 0xFFFFFFFFFFFFFFFF))

    def set_stream(self, stream_ptr: int) -> None:
        self._check(self.lib.esp_set_stream(self.h, C.c_void_p(stream_ptr)))

    # -- hot path ---------------------------------------------------------------
    @staticmethod
    def _opts(mode: int, tilt: float, seed: int, phase: int) -> SweepOpts:
        o = SweepOpts()
        o.mcarlo_mode, o.tilt_angles_max, o.seed, o.phase = int(mode), float(tilt), int(seed) & (2 ** 64 - 1), int(phase)
        return o

    def sweep(self, n: int, first_sweep: int, seed: int, mode: int = 0, tilt: float = 0.125, phase: int = 1):
        o = self._opts(mode, tilt, seed, phase)
        self._check(self.lib.esp_sweep(self.h, int(n), int(first_sweep), C.byref(o)))

    def sweep_colour(self, colour: int, sweep: int, seed: int, mode: int = 0, tilt: float = 0.125, phase: int = 1):
        o = self._opts(mode, tilt, seed, phase)
        self._check(self.lib.esp_sweep_colour(self.h, int(colour), int(sweep), C.byref(o)))

    def pt_swap(self, start: int, swap_index: int, seed: int):
        self._check(self.lib.esp_pt_swap(self.h, int(start), int(swap_index), int(seed) & (2 ** 64 - 1)))

    def schedule(self, steps_warmup: int, steps_mc: int, steps_measure: int, pt: bool = False,
                 pt_steps_swap: int = 1, mode: int = 0, tilt: float = 0.125, seed: int = 1,
                 binning_level=None) -> Schedule:
        s = Schedule()
        s.steps_warmup, s.steps_mc, s.steps_measure = int(steps_warmup), int(steps_mc), int(steps_measure)
        s.pt, s.mcarlo_mode, s.pt_steps_swap = int(bool(pt)), int(mode), int(pt_steps_swap)
        s.tilt_angles_max, s.seed = float(tilt), int(seed) & (2 ** 64 - 1)
        bl = np.ascontiguousarray(binning_level if binning_level else [], dtype=np.int32)
        s.lbinerror = int(bl.size > 0)
        s.num_binning_level = int(bl.size)
        s.binning_level = _p(bl) if bl.size else None
        s._levels = bl  # keep the array alive with the struct
        return s

    def _results(self, nlev: int):
        R = self.R
        out = {
            "rejected": np.zeros((R, 2), dtype=np.int64), "steps_tot": np.zeros(2, dtype=np.int64),
            "energy": np.zeros((R, 3)), "data": np.zeros((R, 6)), "pm": np.zeros((R, self.num_freq())),
            "binning": np.zeros((R, max(nlev, 1), 2)), "num_swaps": np.zeros((R, 2), dtype=np.int64),
            "map": np.zeros(R, dtype=np.int32),
        }
        r = Results()
        for k in ("rejected", "steps_tot", "energy", "data", "pm", "binning", "num_swaps", "map"):
            setattr(r, k, _p(out[k]))
        return out, r

    def begin(self, sched: Schedule) -> None:
        self._sched = sched
        self._check(self.lib.esp_begin(self.h, C.byref(sched)))

    def advance(self, n: int) -> None:
        self._check(self.lib.esp_advance(self.h, int(n)))

    def collect(self) -> dict:
        nlev = self._sched.num_binning_level
        out, r = self._results(nlev)
        self._check(self.lib.esp_collect(self.h, C.byref(r)))
        out["steps_mc_eff"] = r.steps_mc_eff
        if nlev == 0:
            out["binning"] = None
        self._collect_obs(out, nlev)
        return out

    def set_observables(self, order_axes=None, staggered_coeff=None) -> None:
        """Measure the order parameter (order_axes: (num_atoms, 3) unit vectors)
        and / or the staggered magnetisation (staggered_coeff: num_atoms of +1/-1)
        with every measurement; None for both switches them off."""
        flags = (OBS_ORDER_PARAMETER if order_axes is not None else 0) | \
                (OBS_STAGGERED if staggered_coeff is not None else 0)
        ax = np.ascontiguousarray(order_axes, dtype=np.float64).reshape(-1) if order_axes is not None else None
        cf = np.ascontiguousarray(staggered_coeff, dtype=np.int32).reshape(-1) if staggered_coeff is not None else None
        if ax is not None and ax.size != 3 * self.na:
            raise ValueError("order_axes must hold num_atoms x 3 values")
        if cf is not None and cf.size != self.na:
            raise ValueError("staggered_coeff must hold num_atoms values")
        self._check(self.lib.esp_set_observables(self.h, flags, _p(ax) if ax is not None else None,
                                                 _p(cf) if cf is not None else None))
        self._obs = flags

    def set_spin_correlation(self, shells) -> None:
        """Measure spincorr_get with every measurement over the neighbour shells
        of espins_gb300.tables.build_shells (None switches it off)."""
        if shells is None:
            self._check(self.lib.esp_set_spin_correlation(self.h, 0, 1, 0, None, None, None, None))
            self._sc = None
            return
        S, nsp = int(shells.nn.shape[0]), int(shells.count.shape[1])
        maxk = int(shells.nb.shape[1])
        # the reference's Fortran arrays: column-major, 1-based
        kind = np.ascontiguousarray(shells.kind + 1, dtype=np.int32)
        nn = np.asfortranarray(shells.nn.astype(np.int32))                                # (S, N)
        nb = np.asfortranarray(np.transpose(shells.nb, (0, 2, 1)).astype(np.int32) + 1)  # (S, N, maxk)
        cnt = np.asfortranarray(shells.count.astype(np.int32))                            # (S, nsp, nsp)
        self._check(self.lib.esp_set_spin_correlation(self.h, S, nsp, maxk, _p(kind), _p(nn), _p(nb), _p(cnt)))
        self._sc = (S, nsp)

    def set_structure_factor(self, qpts, polar, steps_measure: int, real_lattice, positions) -> None:
        """Measure mcarlo_structure_factor every steps_measure measurements at the
        cartesian q-points qpts (nq, 3); real_lattice rows are a_j, positions
        (N, 3) the cartesian site positions (espins_gb300.tables).  qpts None
        switches it off."""
        if qpts is None:
            self._check(self.lib.esp_set_structure_factor(self.h, 0, None, None, 1, None, None))
            self._sf = 0
            return
        q = np.ascontiguousarray(qpts, dtype=np.float64).reshape(-1, 3)
        p = np.ascontiguousarray(polar, dtype=np.float64).reshape(3)
        rl = np.asfortranarray(np.asarray(real_lattice, dtype=np.float64))        # real_lattice(j, :) = a_j
        pos = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)    # atoms_supercell_pos_cart(3, N)
        self._check(self.lib.esp_set_structure_factor(self.h, q.shape[0], _p(q), _p(p), int(steps_measure),
                                                      _p(rl), _p(pos)))
        self._sf = q.shape[0]

    def _collect_obs(self, out: dict, nlev: int) -> None:
        if getattr(self, "_sf", 0):
            sf = np.zeros((self.R, self._sf, 3))
            n = C.c_int64()
            self._check(self.lib.esp_collect_structure_factor(self.h, _p(sf), C.byref(n)))
            out["sfactor"], out["sfactor_count"] = sf, n.value
        if getattr(self, "_sc", None):
            S, nsp = self._sc
            sc = [np.zeros((self.R, S, nsp, nsp)) for _ in range(3)]
            self._check(self.lib.esp_collect_spin_correlation(self.h, _p(sc[0]), _p(sc[1]), _p(sc[2])))
            out["spincorr"], out["spincorr_abs"], out["spincorr_tot"] = sc
        if not getattr(self, "_obs", 0):
            return
        R, nf = self.R, self.num_freq()
        o = {"obs_data": np.zeros((R, 6)), "pm_op": np.zeros((R, nf)), "pm_sm": np.zeros((R, nf)),
             "obs_binning": np.zeros((R, max(nlev, 1), 2))}
        r = ObsResults()
        r.data, r.pm_op, r.pm_sm, r.binning = (_p(o[k]) for k in ("obs_data", "pm_op", "pm_sm", "obs_binning"))
        self._check(self.lib.esp_collect_observables(self.h, C.byref(r)))
        if not self._obs & OBS_ORDER_PARAMETER:
            o["pm_op"] = None
        if not self._obs & OBS_STAGGERED:
            o["pm_sm"] = None
        if nlev == 0:
            o["obs_binning"] = None
        out.update(o)

    def run(self, steps_warmup: int, steps_mc: int, steps_measure: int, pt: bool = False,
            pt_steps_swap: int = 1, mode: int = 0, tilt: float = 0.125, seed: int = 1,
            binning_level=None) -> dict:
        """esp_run: the whole schedule of mcarlo_main / pt_main."""
        s = self.schedule(steps_warmup, steps_mc, steps_measure, pt, pt_steps_swap, mode, tilt, seed,
                          binning_level)
        nlev = s.num_binning_level
        out, r = self._results(nlev)
        self._check(self.lib.esp_run(self.h, C.byref(s), C.byref(r)))
        out["steps_mc_eff"] = r.steps_mc_eff
        if nlev == 0:
            out["binning"] = None
        self._collect_obs(out, nlev)
        return out

    # -- observables --------------------------------------------------------------
    def energy(self) -> np.ndarray:
        e = np.zeros(self.R)
        self._check(self.lib.esp_energy(self.h, _p(e)))
        return e

    def running_energy(self) -> np.ndarray:
        e = np.zeros(self.R)
        self._check(self.lib.esp_running_energy(self.h, _p(e)))
        return e

    def running_magnetization(self) -> np.ndarray:
        m = np.zeros((self.R, 3))
        self._check(self.lib.esp_running_magnetization(self.h, _p(m)))
        return m

    def local_terms(self):
        g = np.zeros((self.R, self.n, 3))
        q = np.zeros((self.R, self.n, 6))
        self._check(self.lib.esp_local_terms(self.h, _p(g), _p(q)))
        return g, q

    def get_spins(self) -> np.ndarray:
        s = np.zeros((self.R, self.n, 3))
        self._check(self.lib.esp_get_spins(self.h, _p(s)))
        return s

    def colouring(self):
        c = np.zeros(self.n, dtype=np.int32)
        k = C.c_int32()
        self._check(self.lib.esp_get_colouring(self.h, _p(c), C.byref(k)))
        return c, k.value

    def rejected(self) -> np.ndarray:
        r = np.zeros((self.R, 2), dtype=np.int64)
        self._check(self.lib.esp_get_rejected(self.h, _p(r)))
        return r

    def replica_of_slot(self) -> np.ndarray:
        r = np.zeros(self.R, dtype=np.int32)
        self._check(self.lib.esp_get_replica_of_slot(self.h, _p(r)))
        return r

    def set_series(self, capacity: int) -> None:
        self._check(self.lib.esp_set_series(self.h, int(capacity)))

    def series(self) -> np.ndarray:
        """(measurements, R, 2): E and |m| per measurement and temperature slot."""
        n = C.c_int64()
        self._check(self.lib.esp_get_series(self.h, None, C.byref(n)))
        out = np.zeros((n.value, self.R, 2))
        if n.value:
            self._check(self.lib.esp_get_series(self.h, _p(out), C.byref(n)))
        return out

    def set_sweep_kernel(self, kind: str) -> None:
        """'auto', 'ell' (any lattice), 'cluster' (translation-invariant, cluster-resident)
        or 'tile' (translation-invariant, tiles with frozen halos)."""
        k = {"auto": 0, "ell": 1, "cluster": 2, "tile": 4}[kind]
        self._check(self.lib.esp_set_sweep_kernel(self.h, k))

    def sweep_kernel(self):
        """('ell' | 'cluster' | 'learned', cluster size)."""
        k, cs = C.c_int32(), C.c_int32()
        self._check(self.lib.esp_get_sweep_kernel(self.h, C.byref(k), C.byref(cs)))
        return {1: "ell", 2: "cluster", 3: "learned", 4: "tile"}[k.value], cs.value

    # -- learned proposal -----------------------------------------------------
    def lp_init(self, seed: int = 0) -> None:
        self._check(self.lib.esp_lp_init_weights(self.h, int(seed)))

    def lp_set_weights(self, params: np.ndarray) -> None:
        p = np.ascontiguousarray(params, dtype=np.float32)
        if p.size != LP_NUM_PARAMS:
            raise ValueError(f"expected {LP_NUM_PARAMS} parameters")
        self._check(self.lib.esp_lp_set_weights(self.h, _p(p)))

    def lp_weights(self) -> np.ndarray:
        p = np.zeros(LP_NUM_PARAMS, dtype=np.float32)
        self._check(self.lib.esp_lp_get_weights(self.h, _p(p)))
        return p

    def lp_reserve(self, capacity: int) -> None:
        self._check(self.lib.esp_lp_reserve(self.h, int(capacity)))

    def lp_collect(self, colour: int) -> int:
        n = C.c_int64()
        self._check(self.lib.esp_lp_collect(self.h, int(colour), C.byref(n)))
        return n.value

    def lp_data(self, first: int, n: int):
        f = np.zeros((n, LP_IN), dtype=np.float32)
        t = np.zeros((n, 4), dtype=np.float32)
        self._check(self.lib.esp_lp_get_data(self.h, int(first), int(n), _p(f), _p(t)))
        return f, t

    def lp_train(self, steps: int, batch: int = 4096, lr: float = 1e-3, beta1: float = 0.9,
                 beta2: float = 0.999, eps: float = 1e-8, seed: int = 0) -> np.ndarray:
        o = LpTrainOpts(int(steps), int(batch), float(lr), float(beta1), float(beta2), float(eps), int(seed))
        loss = np.zeros(max(1, int(steps)))
        self._check(self.lib.esp_lp_train(self.h, C.byref(o), _p(loss)))
        return loss[:steps]

    def lp_loss_grad(self, features: np.ndarray, targets: np.ndarray):
        f = np.ascontiguousarray(features, dtype=np.float32).reshape(-1, LP_IN)
        t = np.ascontiguousarray(targets, dtype=np.float32).reshape(-1, 4)
        g = np.zeros(LP_NUM_PARAMS, dtype=np.float32)
        loss = C.c_double()
        self._check(self.lib.esp_lp_loss_grad(self.h, _p(f), _p(t), f.shape[0], C.byref(loss), _p(g)))
        return loss.value, g

    def lp_forward(self, features: np.ndarray) -> np.ndarray:
        f = np.ascontiguousarray(features, dtype=np.float32).reshape(-1, LP_IN)
        out = np.zeros((f.shape[0], LP_OUT), dtype=np.float32)
        self._check(self.lib.esp_lp_forward(self.h, _p(f), f.shape[0], _p(out)))
        return out

    def set_cluster_geometry(self, cluster_size: int, threads: int, sites_per_thread: int = 1) -> None:
        self._check(self.lib.esp_set_cluster_geometry(self.h, int(cluster_size), int(threads), int(sites_per_thread)))

    def cluster_geometry(self):
        """(CTAs per replica, threads per CTA, sites per thread) of the cluster
        path, (0, 0, 0) without one."""
        a, b, s = C.c_int32(), C.c_int32(), C.c_int32()
        self._check(self.lib.esp_get_cluster_geometry(self.h, C.byref(a), C.byref(b), C.byref(s)))
        return a.value, b.value, s.value

    def set_tile_geometry(self, tile: int, replicas: int, variant: int = 0) -> None:
        """variant 0: one CTA per tile; persistent pipelined CTAs, 1: one per
        SM, 2: two per SM."""
        self._check(self.lib.esp_set_tile_geometry(self.h, int(tile), int(replicas), int(variant)))

    def set_host_transfer(self, mode: int) -> None:
        """Spin transfers: bit 0 esp_set_spins, bit 1 esp_get_spins read /
        write the caller's array from the device directly (a set bit) or go
        through the pinned staging; -1 the default."""
        self._check(self.lib.esp_set_host_transfer(self.h, int(mode)))

    def host_transfer(self):
        """(mode in effect, whether the device reads and writes pageable host memory)."""
        m, d = C.c_int32(), C.c_int32()
        self._check(self.lib.esp_get_host_transfer(self.h, C.byref(m), C.byref(d)))
        return m.value, bool(d.value)

    def tile_geometry(self):
        """(tile edge in cells, replicas per CTA, variant) of the tiled path, (0, 0, 0) without one."""
        a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
        self._check(self.lib.esp_get_tile_geometry(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def set_pt_groups(self, group_size: int) -> None:
        """Replica exchange only inside consecutive groups of `group_size`
        temperature slots (independent lattices of one shape in one handle)."""
        self._check(self.lib.esp_set_pt_groups(self.h, int(group_size)))

    def lp_set_engine(self, engine: str) -> None:
        """'mma' (warp-level mma.sync) or 'tcgen05' (tensor-memory MMAs on 128-trial tiles)."""
        self._check(self.lib.esp_lp_set_engine(self.h, {"mma": 0, "tcgen05": 1}[engine]))

    def lp_force_tc_timeout(self, on: bool) -> None:
        """Test hook: tcgen05 completion waits report a give-up (see the header)."""
        self._check(self.lib.esp_lp_force_tc_timeout(self.h, int(bool(on))))

    def set_proposal(self, kind: str) -> None:
        """'plain' (the reference's trial moves) or 'learned'."""
        self._check(self.lib.esp_set_proposal(self.h, {"plain": 0, "learned": 1}[kind]))

    def proposal(self) -> str:
        k = C.c_int32()
        self._check(self.lib.esp_get_proposal(self.h, C.byref(k)))
        return ("plain", "learned")[k.value]

    def num_freq(self) -> int:
        k = C.c_int32()
        self._check(self.lib.esp_num_freq(self.h, C.byref(k)))
        return k.value

    def launch_count(self) -> int:
        k = C.c_int64()
        self._check(self.lib.esp_launch_count(self.h, C.byref(k)))
        return k.value


class Batch:
    """Handles advanced together by replayed CUDA graphs (``esp_batch``)."""

    def __init__(self, engines, stream_ptr: int = 0):
        self.lib = load()
        self.engines = list(engines)
        arr = (C.c_void_p * len(self.engines))(*[e.h.value for e in self.engines])
        self._arr = arr
        b = C.c_void_p()
        rc = self.lib.esp_batch_create(arr, len(self.engines), C.c_void_p(stream_ptr), C.byref(b))
        if rc != ESP_OK:
            raise EspError(rc, last_global_error())
        self.b = b

    def _check(self, rc: int):
        if rc != ESP_OK:
            buf = C.create_string_buffer(1024)
            self.lib.esp_batch_last_error(self.b, buf, 1024)
            raise EspError(rc, buf.value.decode())

    def close(self):
        if getattr(self, "b", None):
            self.lib.esp_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_units_per_graph(self, units: int) -> None:
        self._check(self.lib.esp_batch_set_units_per_graph(self.b, int(units)))

    def advance(self, units: int) -> None:
        self._check(self.lib.esp_batch_advance(self.b, int(units)))

    def tune(self, units: int = 2) -> dict:
        n = len(self.engines)
        kern = np.zeros(n, dtype=np.int32)
        ell = np.zeros(n)
        clu = np.zeros(n)
        gr = np.zeros(4)
        cs = np.zeros(n, dtype=np.int32)
        nt = np.zeros(n, dtype=np.int32)
        sp = np.zeros(n, dtype=np.int32)
        t = BatchTuning(0, 0.0, _p(kern), _p(ell), _p(clu), _p(gr), _p(cs), _p(nt), _p(sp))
        self._check(self.lib.esp_batch_tune(self.b, int(units), C.byref(t)))
        return {"units_per_graph": t.units_per_graph, "us_per_unit": t.us_per_unit,
                "kernel": [{1: "ell", 2: "cluster", 4: "tile"}.get(int(k), "ell") for k in kern],
                "ell_us": ell.tolist(),
                "cluster_us": clu.tolist(), "graph_us": dict(zip((1, 2, 4, 8), gr.tolist())),
                "cluster_geometry": [(int(a), int(b), int(c)) for a, b, c in zip(cs, nt, sp)]}
