"""Host driver: what mc_prog does between param_read and the end of the run.

``run(inp)`` mirrors ESpinS's ``mcarlo_main`` (src/mcarlo.F90:62-238) and
``pt_main`` (src/pt.F90:63-500): it builds the tables (jij_get etc.), sets up
the start configuration (mcarlo.F90:271-322, pt.F90:442-491), runs the whole
schedule on the GPU through the C ABI, and writes the reference's output
files.  Differences from the reference, by design:

* temperatures of plain Metropolis run as independent chains from the start
  configuration (the reference chains a rank's temperatures one after the
  other, mcarlo.F90:490-505); stationary statistics are the same;
* the random stream is Philox4x32-10 keyed by one 64-bit seed instead of one
  MT19937 stream per MPI rank;
* sites are updated colour class by colour class instead of in typewriter
  order.
The order parameter, the staggered magnetisation and the spin correlations
(order_parameter, staggered_m, spin_correlation) are measured on the GPU with
every measurement and written to _op.dat / _staggered.dat / _spincorr.dat and
the extra _pm.dat / _binerror.dat columns.  With energy_write the running
energy of every measurement is recorded on the device and written to the
_energy-T###.dat files in chunks of the measurements that fit the device
series buffer.  With sfactor the structure factor is measured every
sfactor_steps_measure measurements and written to _sf-T###.dat (the plotting
scripts _sf.py / _sf.gnu that the reference writes beside them are not).
"""
from __future__ import annotations

import os
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import writers as W
from .lib import Engine
from .mcin import McInput, McinError
from .tables import Hamiltonian, build_hamiltonian, build_shells, sfactor_qpoints, site_positions

UNSUPPORTED = []

# bytes of device memory the energy series may hold at once
SERIES_BYTES = 1 << 28


@dataclass
class RunResult:
    tems: np.ndarray
    res: dict
    spins: np.ndarray
    ham: Hamiltonian
    seed: int


def choose_seed(inp: McInput, seed: Optional[int]) -> int:
    if seed is not None:
        return int(seed) & (2 ** 64 - 1)
    if inp.seeds:
        return int(inp.seeds[0]) & (2 ** 64 - 1)
    return int.from_bytes(os.urandom(8), "little")


def run(inp: McInput, seed: Optional[int] = None, outdir: Optional[str] = None,
        engine_factory=Engine, write: bool = True) -> RunResult:
    for attr, key in UNSUPPORTED:
        if getattr(inp, attr):
            raise McinError(f"{key}: this optional measurement is not part of the GPU Monte Carlo path")
    ham = build_hamiltonian(inp)
    seed = choose_seed(inp, seed)
    R = inp.tems_num
    tems = np.asarray(inp.tems, dtype=float)
    mode = 1 if inp.mcarlo_mode.startswith("const") else 0
    with engine_factory(ham.n, ham.num_atoms, ham.supercell, R, inp.boundary_open) as e:
        e.upload(ham)
        if inp.lorderparam or inp.lstaggered:
            e.set_observables(order_axes=inp.orderparam_axes_cart if inp.lorderparam else None,
                              staggered_coeff=inp.staggered_coeff if inp.lstaggered else None)
        if inp.lspincorr:
            e.set_spin_correlation(build_shells(inp))
        if inp.lsfactor:
            e.set_structure_factor(sfactor_qpoints(inp), inp.sfactor_polar, inp.sfactor_steps_measure,
                                   inp.real_lattice, site_positions(inp))
        e.set_temperatures(tems)
        if inp.initial_sconfig.startswith("file"):
            path = os.path.join(outdir or ".", inp.seedname + "_sconfig.dat")
            s = W.read_sconfig(path, ham.n, tems) * ham.mag[None, :, None]
            e.set_spins(s)
        else:
            e.init_spins("rand" if inp.initial_sconfig.startswith("rand") else "ferro", seed)
        kw = dict(pt=inp.pt, pt_steps_swap=inp.pt_steps_swap, mode=mode, tilt=inp.tilt_angles_max, seed=seed,
                  binning_level=inp.binning_level if inp.lbinerror else None)
        if inp.energy_write and write and outdir is not None:
            res = _run_with_series(e, inp, outdir, tems, ham.n, kw)
        else:
            res = e.run(inp.steps_warmup, inp.steps_mc, inp.steps_measure, **kw)
        spins = e.get_spins()
    out = RunResult(tems=tems, res=res, spins=spins, ham=ham, seed=seed)
    if write and outdir is not None:
        write_outputs(inp, out, outdir)
    return out


def _run_with_series(e: Engine, inp: McInput, outdir: str, tems, n: int, kw) -> dict:
    """esp_begin / esp_advance / esp_collect with the energy series read back
    after every chunk of measurement units (open_E_unit, write_E: the
    reference writes every energy_num_print measurements; the content of the
    files does not depend on the chunking)."""
    R = len(tems)
    per_unit = inp.pt_steps_swap if inp.pt else 1
    units = -(-inp.steps_mc // per_unit) if inp.pt else inp.steps_mc
    nsteps = units * per_unit
    chunk = max(1, min(units, SERIES_BYTES // (16 * R * per_unit)))
    e.set_series(chunk * per_unit)
    os.makedirs(outdir, exist_ok=True)
    series = W.EnergySeries(os.path.join(outdir, inp.seedname or "espins"), tems, nsteps, n)
    try:
        e.begin(e.schedule(inp.steps_warmup, inp.steps_mc, inp.steps_measure, **kw))
        done = 0
        while done < units:
            k = min(chunk, units - done)
            e.advance(k)
            done += k
            series.append(e.series()[-k * per_unit:, :, 0])
        return e.collect()
    finally:
        series.close()
        e.set_series(0)


def write_outputs(inp: McInput, r: RunResult, outdir: str) -> None:
    os.makedirs(outdir, exist_ok=True)
    base = os.path.join(outdir, inp.seedname or "espins")
    n = r.ham.n
    m_max = float(np.abs(inp.mag_cell).sum())
    res = r.res
    op, sm = bool(inp.lorderparam), bool(inp.lstaggered)
    W.write_mc_dat(base + "_mc.dat", r.tems, res["data"], n)
    W.write_pm_dat(base + "_pm.dat", r.tems, res["pm"], -m_max, m_max,
                   pm_op=res.get("pm_op") if op else None, pm_sm=res.get("pm_sm") if sm else None, pt=inp.pt)
    W.write_sconfig(base + "_sconfig.dat", inp.supercell_size, r.tems, r.spins)
    if op:
        W.write_obs_dat(base + "_op.dat", "op", r.tems, res["obs_data"], n)
    if sm:
        W.write_obs_dat(base + "_staggered.dat", "staggered", r.tems, res["obs_data"], n)
    if inp.lsfactor:
        W.write_sfactor(base, r.tems, res["sfactor"],
                        W.sfactor_plane_coords(inp.sfactor_corner, inp.sfactor_q1, inp.sfactor_q2,
                                               inp.sfactor_2dqmesh), inp.lsfactor_polar)
    if inp.lspincorr:
        W.write_spincorr(base + "_spincorr.dat", r.tems, res["spincorr"], res["spincorr_abs"], res["spincorr_tot"],
                         inp.atoms_symbol)
    if inp.lbinerror and res["binning"] is not None:
        W.write_binerror(base + "_binerror.dat", r.tems, res["binning"], inp.binning_level, n, inp.pt,
                         obs_binning=res.get("obs_binning"), op=op, sm=sm)
    with open(base + ".mcout", "w") as fh:
        fh.write(W.mcout_block(r.tems, r.res, n, inp.pt))
