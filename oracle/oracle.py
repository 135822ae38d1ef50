"""ctypes front end of the FP64 CPU oracle (``espins_oracle.c``).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA library.  Only tests/,
``__graft_entry__.smoke()`` and bench.py's CPU baseline arm may import it.

Every function mirrors one routine of the reference (ESpinS, Fortran 90);
the file:line anchors are in ``espins_oracle.c``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    srcs = [os.path.join(HERE, f) for f in ("espins_oracle.c", "lp_oracle.c", "Makefile")]
    if force or not os.path.exists(LIB_PATH) or any(os.path.getmtime(LIB_PATH) < os.path.getmtime(s) for s in srcs):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


class OrMt(C.Structure):
    _fields_ = [("mti", C.c_int32), ("mt", C.c_uint32 * 624)]


class OrHam(C.Structure):
    _fields_ = [
        ("n", C.c_int32), ("num_atoms", C.c_int32), ("mag", C.c_void_p),
        ("j_maxnb", C.c_int32), ("j_nn", C.c_void_p), ("j_nb", C.c_void_p), ("j_val", C.c_void_p),
        ("b_maxnb", C.c_int32), ("b_nn", C.c_void_p), ("b_nb", C.c_void_p), ("b_val", C.c_void_p),
        ("d_maxnb", C.c_int32), ("d_nn", C.c_void_p), ("d_nb", C.c_void_p), ("d_val", C.c_void_p),
        ("have_si", C.c_int32), ("si_axis", C.c_void_p), ("si_delta", C.c_void_p),
        ("have_field", C.c_int32), ("f_axis", C.c_void_p), ("f_val", C.c_void_p),
    ]


class OrMcOpts(C.Structure):
    _fields_ = [("steps_warmup", C.c_int64), ("steps_mc", C.c_int64), ("steps_measure", C.c_int64),
                ("mode", C.c_int32), ("tilt", C.c_double),
                ("num_binning_level", C.c_int32), ("binning_level", C.c_void_p)]


class OrShells(C.Structure):
    _fields_ = [("num_shells", C.c_int32), ("num_species", C.c_int32), ("maxk", C.c_int32),
                ("kind", C.c_void_p), ("nn", C.c_void_p), ("nb", C.c_void_p), ("count", C.c_void_p)]


class OrObs(C.Structure):
    _fields_ = [("op_axes", C.c_void_p), ("st_coeff", C.c_void_p), ("data", C.c_void_p),
                ("pm_op", C.c_void_p), ("pm_st", C.c_void_p), ("binning", C.c_void_p),
                ("shells", C.c_void_p), ("sc", C.c_void_p), ("sc_abs", C.c_void_p), ("sc_tot", C.c_void_p)]


class OrMcResult(C.Structure):
    _fields_ = [("rejected", C.c_int64 * 2), ("steps_tot", C.c_int64 * 2),
                ("energy", C.c_double * 3), ("data", C.c_double * 6),
                ("pm", C.c_void_p), ("binning", C.c_void_p), ("obs", C.c_void_p)]


class OrPtOpts(C.Structure):
    _fields_ = [("steps_warmup", C.c_int64), ("steps_mc", C.c_int64), ("steps_measure", C.c_int64),
                ("pt_steps_swap", C.c_int64), ("mode", C.c_int32), ("tilt", C.c_double),
                ("num_binning_level", C.c_int32), ("binning_level", C.c_void_p)]


class OrPtResult(C.Structure):
    _fields_ = [("rejected", C.c_void_p), ("num_swaps", C.c_void_p), ("map", C.c_void_p),
                ("energy", C.c_void_p), ("data", C.c_void_p), ("pm", C.c_void_p),
                ("binning", C.c_void_p), ("obs", C.c_void_p), ("steps_mc_eff", C.c_int64),
                ("steps_tot_main", C.c_int64)]


def _declare(L):
    P = C.POINTER
    L.or_mt_init.argtypes = [P(OrMt), C.c_int32]
    L.or_mt_u32.argtypes = [P(OrMt)]
    L.or_mt_u32.restype = C.c_uint32
    L.or_mt_real2.argtypes = [P(OrMt)]
    L.or_mt_real2.restype = C.c_double
    L.or_philox4x32_10.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    L.or_energy.argtypes = [P(OrHam), C.c_void_p]
    L.or_energy.restype = C.c_double
    L.or_delta_energy.argtypes = [P(OrHam), C.c_int, C.c_void_p, C.c_void_p]
    L.or_delta_energy.restype = C.c_double
    L.or_local_terms.argtypes = [P(OrHam), C.c_void_p, C.c_void_p, C.c_void_p]
    L.or_metropolis.argtypes = [P(OrHam), P(OrMt), C.c_int, C.c_double, C.c_void_p,
                                P(C.c_double), P(C.c_int64), C.c_int, C.c_double]
    L.or_magnetization2.argtypes = [P(OrHam), C.c_void_p]
    L.or_magnetization2.restype = C.c_double
    L.or_num_freq.argtypes = [P(OrHam)]
    L.or_num_freq.restype = C.c_int
    L.or_pm.argtypes = [P(OrHam), C.c_void_p, C.c_int, C.c_void_p]
    L.or_mcarlo_run.argtypes = [P(OrHam), P(OrMcOpts), P(OrMt), C.c_double, C.c_void_p, P(OrMcResult)]
    L.or_pt_run.argtypes = [P(OrHam), P(OrPtOpts), P(OrMt), C.c_int, C.c_void_p, C.c_void_p, P(OrPtResult)]
    L.or_trial_spin.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_double, C.c_void_p, C.c_void_p]
    L.or_colour_pass_philox.argtypes = [P(OrHam), C.c_void_p, C.c_int, C.c_double, C.c_void_p,
                                        C.c_int, C.c_uint64, C.c_uint64, C.c_int, C.c_double,
                                        P(C.c_double), C.c_void_p, C.c_void_p]
    L.or_colour_pass_philox.restype = C.c_int64
    L.or_build_ell.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                               C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                               C.c_void_p, C.c_void_p, C.c_void_p, P(C.c_int32)]
    L.or_build_ell.restype = C.c_int
    L.or_orderparam2.argtypes = [P(OrHam), C.c_void_p, C.c_void_p]
    L.or_orderparam2.restype = C.c_double
    L.or_staggered2.argtypes = [P(OrHam), C.c_void_p, C.c_void_p]
    L.or_staggered2.restype = C.c_double
    L.or_pm_obs.argtypes = [P(OrHam), C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.or_spincorr.argtypes = [P(OrHam), P(OrShells), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.or_structure_factor.argtypes = [P(OrHam), C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p]
    L.or_lp_num_params.restype = C.c_int
    L.or_lp_forward.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
    L.or_lp_loss_grad.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
    L.or_lp_loss_grad.restype = C.c_double
    L.or_vmf_logpdf.argtypes = [C.c_void_p, C.c_double, C.c_void_p]
    L.or_vmf_logpdf.restype = C.c_double
    L.or_vmf_sample.argtypes = [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p]
    L.or_lp_features.argtypes = [C.c_double, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                 P(C.c_double), C.c_void_p]


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class MT:
    """MT19937 seeded the way ``mtprng_init`` seeds it."""

    def __init__(self, seed: int):
        self.st = OrMt()
        lib().or_mt_init(C.byref(self.st), int(np.int32(seed)))

    def u32(self) -> int:
        return lib().or_mt_u32(C.byref(self.st))

    def real2(self) -> float:
        return lib().or_mt_real2(C.byref(self.st))


def philox4x32_10(ctr, key):
    c = np.asarray(ctr, dtype=np.uint32).copy()
    k = np.asarray(key, dtype=np.uint32).copy()
    out = np.zeros(4, dtype=np.uint32)
    lib().or_philox4x32_10(_ptr(c), _ptr(k), _ptr(out))
    return out


class Ham:
    """Holds contiguous numpy copies of the ELL tables and an ``or_ham`` view.

    Takes the product's Hamiltonian-like object (attributes n, num_atoms, mag,
    jij/bij/dij with nn/nb/val, si_axis/si_delta, field_axis/field_val) or the
    same data as keyword arguments.
    """

    def __init__(self, h):
        self._keep = []
        s = OrHam()
        s.n = int(h.n)
        s.num_atoms = int(h.num_atoms)
        s.mag = self._arr(h.mag, np.float64)
        s.j_maxnb, s.j_nn, s.j_nb, s.j_val = self._ell(h.jij, 1)
        if getattr(h, "bij", None) is not None:
            s.b_maxnb, s.b_nn, s.b_nb, s.b_val = self._ell(h.bij, 1)
        if getattr(h, "dij", None) is not None:
            s.d_maxnb, s.d_nn, s.d_nb, s.d_val = self._ell(h.dij, 3)
        if getattr(h, "si_axis", None) is not None:
            s.have_si = 1
            s.si_axis = self._arr(h.si_axis, np.float64)
            s.si_delta = self._arr(h.si_delta, np.float64)
        if getattr(h, "field_axis", None) is not None:
            s.have_field = 1
            s.f_axis = self._arr(h.field_axis, np.float64)
            s.f_val = self._arr(h.field_val, np.float64)
        self.s = s
        self.n = s.n

    def _arr(self, a, dt):
        a = np.ascontiguousarray(a, dtype=dt)
        self._keep.append(a)
        return a.ctypes.data

    def _ell(self, t, vdim):
        nn = self._arr(t.nn, np.int32)
        nb = self._arr(t.nb, np.int32)
        val = self._arr(t.val, np.float64)
        return int(t.nb.shape[0]), nn, nb, val

    @property
    def ref(self):
        return C.byref(self.s)

    # -- routines -----------------------------------------------------------
    def energy(self, spins: np.ndarray) -> float:
        s = np.ascontiguousarray(spins, dtype=np.float64)
        return lib().or_energy(self.ref, _ptr(s))

    def local_terms(self, spins: np.ndarray):
        s = np.ascontiguousarray(spins, dtype=np.float64)
        g = np.zeros((self.n, 3))
        q = np.zeros((self.n, 6))
        lib().or_local_terms(self.ref, _ptr(s), _ptr(g), _ptr(q))
        return g, q

    def magnetization2(self, spins) -> float:
        s = np.ascontiguousarray(spins, dtype=np.float64)
        return lib().or_magnetization2(self.ref, _ptr(s))

    def num_freq(self) -> int:
        return lib().or_num_freq(self.ref)

    def orderparam2(self, axes, spins) -> float:
        a = np.ascontiguousarray(axes, dtype=np.float64)
        s = np.ascontiguousarray(spins, dtype=np.float64)
        return lib().or_orderparam2(self.ref, _ptr(a), _ptr(s))

    def staggered2(self, coeff, spins) -> float:
        c = np.ascontiguousarray(coeff, dtype=np.float64)
        s = np.ascontiguousarray(spins, dtype=np.float64)
        return lib().or_staggered2(self.ref, _ptr(c), _ptr(s))

    def pm_obs(self, spins, axes=None, coeff=None):
        """P(OP) and P(SM) hits of one configuration (Pm_get's optional parts)."""
        nf = self.num_freq()
        s = np.ascontiguousarray(spins, dtype=np.float64)
        a = np.ascontiguousarray(axes, dtype=np.float64) if axes is not None else None
        c = np.ascontiguousarray(coeff, dtype=np.float64) if coeff is not None else None
        po = np.zeros(nf) if a is not None else None
        ps = np.zeros(nf) if c is not None else None
        lib().or_pm_obs(self.ref, _ptr(s), nf, _ptr(a) if a is not None else None,
                        _ptr(c) if c is not None else None,
                        _ptr(po) if po is not None else None, _ptr(ps) if ps is not None else None)
        return po, ps

    def _shells(self, sh):
        """An or_shells view of a ShellTables-like object (kind, nn, nb, count)."""
        o = OrShells()
        o.num_shells, o.num_species, o.maxk = int(sh.nn.shape[0]), int(sh.count.shape[1]), int(sh.nb.shape[1])
        o.kind = self._arr(sh.kind, np.int32)
        o.nn = self._arr(sh.nn, np.int32)
        o.nb = self._arr(sh.nb, np.int32)
        o.count = self._arr(sh.count, np.int32)
        self._keep.append(o)
        return o

    def spincorr(self, shells, spins):
        """One spincorr_get call: (sum, sum of |.|, |sum|) per shell and species pair."""
        o = self._shells(shells)
        B = (o.num_shells, o.num_species, o.num_species)
        out = [np.zeros(B) for _ in range(3)]
        s = np.ascontiguousarray(spins, dtype=np.float64)
        lib().or_spincorr(self.ref, C.byref(o), _ptr(s), _ptr(out[0]), _ptr(out[1]), _ptr(out[2]))
        return out[0], out[1], out[2]

    def _obs(self, R, nlev, op_axes, st_coeff, want_pm, shells=None):
        """An or_obs for R slots, or (None, None) when no optional measurement is on."""
        if op_axes is None and st_coeff is None and shells is None:
            return None, None
        nf = self.num_freq()
        out = {"obs_data": np.zeros((R, 6)),
               "pm_op": np.zeros((R, nf)) if want_pm and op_axes is not None else None,
               "pm_st": np.zeros((R, nf)) if want_pm and st_coeff is not None else None,
               "obs_binning": np.zeros((R, nlev, 2)) if nlev else None}
        ob = OrObs()
        if op_axes is not None:
            ob.op_axes = self._arr(np.asarray(op_axes).reshape(-1), np.float64)
        if st_coeff is not None:
            ob.st_coeff = self._arr(np.asarray(st_coeff).reshape(-1), np.float64)
        ob.data = _ptr(out["obs_data"])
        ob.pm_op = _ptr(out["pm_op"]) if out["pm_op"] is not None else None
        ob.pm_st = _ptr(out["pm_st"]) if out["pm_st"] is not None else None
        ob.binning = _ptr(out["obs_binning"]) if nlev else None
        if shells is not None:
            sh = self._shells(shells)
            B = (R, sh.num_shells, sh.num_species, sh.num_species)
            for k in ("spincorr", "spincorr_abs", "spincorr_tot"):
                out[k] = np.zeros(B)
            ob.shells = C.addressof(sh)
            ob.sc, ob.sc_abs, ob.sc_tot = (_ptr(out[k]) for k in ("spincorr", "spincorr_abs", "spincorr_tot"))
        self._keep.append(ob)
        return ob, out

    def structure_factor(self, pos, qpts, polar, spins, sf=None):
        """mcarlo_structure_factor of one configuration, added to sf (nq, 3)."""
        q = np.ascontiguousarray(qpts, dtype=np.float64)
        if sf is None:
            sf = np.zeros((q.shape[0], 3))
        r = np.ascontiguousarray(pos, dtype=np.float64)
        p = np.ascontiguousarray(polar, dtype=np.float64)
        s = np.ascontiguousarray(spins, dtype=np.float64)
        lib().or_structure_factor(self.ref, _ptr(r), q.shape[0], _ptr(q), _ptr(p), _ptr(s), _ptr(sf))
        return sf

    def pm(self, spins, pdf=None):
        nf = self.num_freq()
        if pdf is None:
            pdf = np.zeros(nf)
        s = np.ascontiguousarray(spins, dtype=np.float64)
        lib().or_pm(self.ref, _ptr(s), nf, _ptr(pdf))
        return pdf

    def metropolis(self, mt: MT, i: int, beta: float, spins: np.ndarray, energy: float,
                   rejected: int = 0, mode: int = 0, tilt: float = 0.125):
        e = C.c_double(energy)
        r = C.c_int64(rejected)
        lib().or_metropolis(self.ref, C.byref(mt.st), i, beta, _ptr(spins), C.byref(e), C.byref(r),
                            mode, tilt)
        return e.value, r.value

    def mcarlo(self, mt: MT, beta: float, spins: np.ndarray, steps_warmup: int, steps_mc: int,
               steps_measure: int, mode: int = 0, tilt: float = 0.125, binning_level=None,
               want_pm: bool = True, op_axes=None, st_coeff=None, shells=None):
        """One temperature chain.  op_axes (num_atoms, 3) unit vectors and
        st_coeff (num_atoms,) switch on the order parameter and the staggered
        magnetisation; their sums, P(OP)/P(SM) hits and binning variances come
        back as obs_data (1, 6), pm_op / pm_st (1, nf) and obs_binning;
        shells (espins_gb300.tables.ShellTables) switches on the spin
        correlations: spincorr / spincorr_abs / spincorr_tot (1, S, nsp, nsp) sums."""
        o = OrMcOpts()
        o.steps_warmup, o.steps_mc, o.steps_measure = steps_warmup, steps_mc, steps_measure
        o.mode, o.tilt = mode, tilt
        bl = np.asarray(binning_level if binning_level is not None else [], dtype=np.int32)
        o.num_binning_level = bl.size
        o.binning_level = _ptr(bl) if bl.size else None
        res = OrMcResult()
        pm = np.zeros(self.num_freq()) if want_pm else None
        bn = np.zeros(2 * bl.size) if bl.size else None
        res.pm = _ptr(pm) if pm is not None else None
        res.binning = _ptr(bn) if bn is not None else None
        ob, obs = self._obs(1, bl.size, op_axes, st_coeff, want_pm, shells)
        res.obs = C.addressof(ob) if ob is not None else None
        lib().or_mcarlo_run(self.ref, C.byref(o), C.byref(mt.st), beta, _ptr(spins), C.byref(res))
        out = {
            "rejected": list(res.rejected), "steps_tot": list(res.steps_tot),
            "energy": list(res.energy), "data": np.array(res.data[:]),
            "pm": pm, "binning": bn.reshape(-1, 2) if bn is not None else None,
        }
        if obs is not None:
            out.update(obs)
        return out

    def pt(self, mt: MT, tems, spins: np.ndarray, steps_warmup: int, steps_mc: int,
           steps_measure: int, pt_steps_swap: int, mode: int = 0, tilt: float = 0.125,
           binning_level=None, want_pm: bool = True, op_axes=None, st_coeff=None, shells=None):
        tems = np.ascontiguousarray(tems, dtype=np.float64)
        R = tems.size
        o = OrPtOpts()
        o.steps_warmup, o.steps_mc, o.steps_measure = steps_warmup, steps_mc, steps_measure
        o.pt_steps_swap, o.mode, o.tilt = pt_steps_swap, mode, tilt
        bl = np.asarray(binning_level if binning_level is not None else [], dtype=np.int32)
        o.num_binning_level = bl.size
        o.binning_level = _ptr(bl) if bl.size else None
        nf = self.num_freq()
        out = {
            "rejected": np.zeros(R, dtype=np.int64), "num_swaps": np.zeros((R, 2), dtype=np.int64),
            "map": np.zeros(R, dtype=np.int32), "energy": np.zeros((R, 3)), "data": np.zeros((R, 6)),
            "pm": np.zeros((R, nf)) if want_pm else None,
            "binning": np.zeros((R, bl.size, 2)) if bl.size else None,
        }
        res = OrPtResult()
        res.rejected = _ptr(out["rejected"]); res.num_swaps = _ptr(out["num_swaps"])
        res.map = _ptr(out["map"]); res.energy = _ptr(out["energy"]); res.data = _ptr(out["data"])
        res.pm = _ptr(out["pm"]) if want_pm else None
        res.binning = _ptr(out["binning"]) if bl.size else None
        ob, obs = self._obs(R, bl.size, op_axes, st_coeff, want_pm, shells)
        res.obs = C.addressof(ob) if ob is not None else None
        if obs is not None:
            out.update(obs)
        lib().or_pt_run(self.ref, C.byref(o), C.byref(mt.st), R, _ptr(tems), _ptr(spins), C.byref(res))
        out["steps_mc_eff"] = res.steps_mc_eff
        out["steps_tot_main"] = res.steps_tot_main
        return out

    def colour_pass_philox(self, colour: np.ndarray, c: int, beta: float, spins: np.ndarray,
                           replica: int, sweep: int, seed: int, mode: int = 0, tilt: float = 0.125):
        col = np.ascontiguousarray(colour, dtype=np.int32)
        acc = np.zeros(self.n, dtype=np.int8)
        de = np.zeros(self.n)
        e = C.c_double(0.0)
        rej = lib().or_colour_pass_philox(self.ref, _ptr(col), c, beta, _ptr(spins), replica,
                                          sweep, seed, mode, tilt, C.byref(e), _ptr(acc), _ptr(de))
        return rej, e.value, acc, de


def build_ell(num_atoms, atoms_frac, mag_cell, supercell, open_boundary, f1, f2, values):
    """The oracle's own pair expansion (jij.F90:196-446) for cross-checking."""
    values = np.ascontiguousarray(values, dtype=np.float64)
    vdim = 3 if values.ndim == 2 else 1
    npairs = f1.shape[0]
    sc = np.ascontiguousarray(supercell, dtype=np.int32)
    n = int(np.prod(sc)) * num_atoms
    nn = np.zeros(n, dtype=np.int32)
    nb = np.zeros(n * npairs, dtype=np.int32)
    val = np.zeros(n * npairs * vdim, dtype=np.float64)
    mx = C.c_int32(0)
    af = np.ascontiguousarray(atoms_frac, dtype=np.float64)
    mc = np.ascontiguousarray(mag_cell, dtype=np.float64)
    f1c = np.ascontiguousarray(f1, dtype=np.float64)
    f2c = np.ascontiguousarray(f2, dtype=np.float64)
    rc = lib().or_build_ell(num_atoms, _ptr(af), _ptr(mc), _ptr(sc), int(open_boundary), npairs,
                            _ptr(f1c), _ptr(f2c), _ptr(values), vdim, _ptr(nn), _ptr(nb), _ptr(val),
                            C.byref(mx))
    if rc != 0:
        raise ValueError(f"or_build_ell: unrecognised position (code {rc})")
    m = mx.value
    nb = nb[: m * n].reshape(m, n)
    val = val[: m * n * vdim].reshape((m, n, 3) if vdim == 3 else (m, n))
    return nn, nb, val


def read_sconfig(path: str):
    """Parse a ``seed_sconfig.dat`` file: returns (supercell, temps, spins[T, N, 3])."""
    with open(path) as fh:
        lines = fh.read().splitlines()
    sc = tuple(int(x) for x in lines[1].split())
    nw, nt = (int(x) for x in lines[2].split())
    temps, spins = [], []
    pos = 3
    for _ in range(nt):
        temps.append(float(lines[pos])); pos += 1
        blk = np.array([[float(v) for v in lines[pos + j].split()] for j in range(nw)])
        spins.append(blk); pos += nw
    return sc, np.array(temps), np.array(spins)


# ---- learned proposal: FP64 network, mixture head and gradient (lp_oracle.c) ----

LP_IN, LP_HID, LP_OUT = 12, 128, 20


def lp_num_params() -> int:
    return int(lib().or_lp_num_params())


def lp_forward(params: np.ndarray, x: np.ndarray) -> np.ndarray:
    p = np.ascontiguousarray(params, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, LP_IN)
    out = np.zeros((x.shape[0], LP_OUT))
    lib().or_lp_forward(_ptr(p), _ptr(x), x.shape[0], _ptr(out))
    return out


def lp_loss_grad(params: np.ndarray, x: np.ndarray, t: np.ndarray):
    """Mean negative log-likelihood of (features, targets) and its gradient."""
    p = np.ascontiguousarray(params, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, LP_IN)
    t = np.ascontiguousarray(t, dtype=np.float64).reshape(-1, 4)
    g = np.zeros(p.size)
    loss = lib().or_lp_loss_grad(_ptr(p), _ptr(x), _ptr(t), x.shape[0], _ptr(g))
    return float(loss), g


def vmf_logpdf(o, kappa0: float, s) -> float:
    o = np.ascontiguousarray(o, dtype=np.float64)
    s = np.ascontiguousarray(s, dtype=np.float64)
    return float(lib().or_vmf_logpdf(_ptr(o), float(kappa0), _ptr(s)))


def vmf_sample(o, kappa0: float, u) -> np.ndarray:
    o = np.ascontiguousarray(o, dtype=np.float64)
    u = np.ascontiguousarray(u, dtype=np.float64)
    s = np.zeros(3)
    lib().or_vmf_sample(_ptr(o), float(kappa0), _ptr(u), _ptr(s))
    return s


def lp_features(beta: float, mag: float, g, q, axis):
    """(frame rows (3,3), kappa0, features (12,)) of one site."""
    g = np.ascontiguousarray(g, dtype=np.float64)
    q = np.ascontiguousarray(q, dtype=np.float64)
    a = np.ascontiguousarray(axis, dtype=np.float64)
    e = np.zeros(9)
    k0 = C.c_double(0.0)
    f = np.zeros(LP_IN)
    lib().or_lp_features(float(beta), float(mag), _ptr(g), _ptr(q), _ptr(a), _ptr(e), C.byref(k0), _ptr(f))
    return e.reshape(3, 3), float(k0.value), f
