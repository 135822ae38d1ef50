"""Synthetic ``.mcin`` inputs with the shapes of the benchmark configurations.

Each function returns the text of an input file in the reference's keyword
format (the same text the reference's mc.x would read), so every workload
goes through the same reader and table builder as a user's input.  Units:
couplings in eV as the reference reads them; single-ion Delta > 0 is easy
plane and Delta < 0 easy axis (+Delta (a.S)^2, get_quant.F90:227-233).
"""
from __future__ import annotations

from typing import Dict, List, Optional, Sequence, Tuple

from .mcin import McInput, parse_mcin

NN = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]
NNN = ([(a, b, 0) for a in (1, -1) for b in (1, -1)] + [(a, 0, b) for a in (1, -1) for b in (1, -1)]
       + [(0, a, b) for a in (1, -1) for b in (1, -1)])
N3 = [(a, b, c) for a in (1, -1) for b in (1, -1) for c in (1, -1)]
BCC1 = [(a * 0.5, b * 0.5, c * 0.5) for a in (1, -1) for b in (1, -1) for c in (1, -1)]


def _fmt(x: float) -> str:
    return repr(float(x))


def lattice_mcin(atoms: Sequence[Tuple[str, Tuple[float, float, float], float]], L: int,
                 exchange: Sequence[Tuple[float, Sequence[Tuple[float, float, float]]]],
                 tems: Optional[Sequence[float]] = None, tems_mode: str = "man",
                 tem_range: Optional[Tuple[float, float, int]] = None,
                 biquad: Optional[Tuple[float, Sequence]] = None,
                 dm: Optional[Tuple[float, Sequence]] = None,
                 single_ion: Optional[float] = None, pt: bool = False, pt_steps_swap: int = 1,
                 steps: Tuple[int, int, int] = (1000, 10000, 1), initial: str = "rand",
                 mode: str = "random", lattice_const: float = 1.0) -> str:
    """Input text for a cubic cell with the given basis and shells.

    exchange: [(J_eV, offsets)]; offsets are fractional vectors applied to every
    basis atom.  biquad/dm: (value_eV, offsets), the DM vector along the unit
    bond vector.
    """
    a = lattice_const
    out: List[str] = ["begin unit_cell_cart", f"{a} 0 0", f"0 {a} 0", f"0 0 {a}", "end unit_cell_cart",
                      "begin atoms_frac"]
    out += [f"{lab} {p[0]} {p[1]} {p[2]} {m}" for lab, p, m in atoms]
    out += ["end atoms_frac", f"supercell_size = {L} {L} {L}"]
    if tems is not None:
        out += ["tems_mode = man", f"tems_num = {len(tems)}", "tems = " + " ".join(_fmt(t) for t in tems)]
    else:
        t0, t1, n = tem_range
        out += [f"tems_mode = {tems_mode}", f"tem_start = {t0}", f"tem_end = {t1}", f"tems_num = {n}"]
    out += [f"steps_warmup = {steps[0]}", f"steps_mc = {steps[1]}", f"steps_measure = {steps[2]}",
            f"initial_sconfig = {initial}", f"mcarlo_mode = {mode}"]
    if pt:
        out += ["pt = .true.", f"pt_steps_swap = {pt_steps_swap}"]

    def pair_block(name, word, value_offsets):
        rows = [f"begin {name}"]
        for val, offs in value_offsets:
            for _, p, _m in atoms:
                for o in offs:
                    rows.append(f"f1={p[0]},{p[1]},{p[2]}:f2={p[0] + o[0]},{p[1] + o[1]},{p[2] + o[2]}:{word}={val}")
        rows.append(f"end {name}")
        return rows

    out += pair_block("jij_parameters", "jij", exchange)
    if biquad is not None:
        out += ["ham_bij = .true."] + pair_block("bij_parameters", "bij", [biquad])
    if dm is not None:
        out += ["ham_dij = .true."] + pair_block("dij_parameters", "dij", [dm])
        out += ["begin dij_vectors_cart"]
        for _ in atoms:
            out += [f"{o[0]} {o[1]} {o[2]}" for o in dm[1]]
        out += ["end dij_vectors_cart"]
    if single_ion is not None:
        labels = []
        for lab, _p, _m in atoms:
            labels.append(lab)
        out += ["ham_singleion = .true.", "begin singleion_axes_cart"]
        out += [f"{lab} 0 0 1 {single_ion}" for lab in labels]
        out += ["end singleion_axes_cart"]
    return "\n".join(out) + "\n"


SC = [("Fe", (0.0, 0.0, 0.0), 1.0)]
BCC = [("Fe", (0.0, 0.0, 0.0), 1.0), ("Fe", (0.5, 0.5, 0.5), 1.0)]

# name -> (description, text builder)
WORKLOADS: Dict[str, str] = {
    "sc16_plain": "plain Metropolis, SC L=16 (4096 spins), J1=+1.0 meV, 20 T linear 5-30 K",
    "bcc24_pt": "parallel tempering, bcc L=24 (27648 spins), J1=+2.0/J2=+0.5/J3=-0.1 meV, "
                "easy-axis 0.05 meV, 48 replicas geometric 10-80 K, swap every 10 sweeps",
    "sc48_frustrated_pt": "PT, SC L=48 (110592 spins), J1=+1.0/J2=-0.6 meV, B=0.05 meV, "
                          "easy-plane 0.2 meV, 32 replicas 2-30 K",
    "sc128_pt": "PT, SC L=128 (2097152 spins) x 64 replicas, J1=+1.0/J2=+0.3/J3=-0.05 meV, "
                "NN DM 0.1 meV along the bond, easy-axis 0.03 meV, 5-40 K",
}


def workload_text(name: str, L: Optional[int] = None, replicas: Optional[int] = None,
                  steps: Tuple[int, int, int] = (1000, 10000, 1)) -> str:
    if name == "sc16_plain":
        return lattice_mcin(SC, L or 16, [(1e-3, NN)], tem_range=(5.0, 30.0, replicas or 20),
                            tems_mode="lin", steps=steps)
    if name == "bcc24_pt":
        return lattice_mcin(BCC, L or 24, [(2e-3, BCC1), (5e-4, NN), (-1e-4, NNN)],
                            tem_range=(10.0, 80.0, replicas or 48), tems_mode="log",
                            single_ion=-5e-5, pt=True, pt_steps_swap=10, steps=steps)
    if name == "sc48_frustrated_pt":
        return lattice_mcin(SC, L or 48, [(1e-3, NN), (-6e-4, NNN)], tem_range=(2.0, 30.0, replicas or 32),
                            tems_mode="log", biquad=(5e-5, NN), single_ion=2e-4, pt=True,
                            pt_steps_swap=10, steps=steps)
    if name == "sc128_pt":
        return lattice_mcin(SC, L or 128, [(1e-3, NN), (3e-4, NNN), (-5e-5, N3)],
                            tem_range=(5.0, 40.0, replicas or 64), tems_mode="log",
                            dm=(1e-4, NN), single_ion=-3e-5, pt=True, pt_steps_swap=10, steps=steps)
    raise KeyError(name)


def workload(name: str, **kw) -> McInput:
    return parse_mcin(workload_text(name, **kw), seedname=name)


# ---------------------------------------------------------------------------
# Many independent lattices: 512 simple-cubic lattices, L drawn uniformly
# from {8, 12, ..., 48} with seed 3, J1 = +1.0 meV, nearest-neighbour
# biquadratic 0.1 meV and DM 0.2 meV along the unit bond vector, 16 PT
# replicas per lattice log-spaced 2-25 K, a swap every 10 sweeps.
# Lattices of one size share their tables, so they become replica groups of
# one handle (esp_set_pt_groups); the sizes are the handles of one batch.
# ---------------------------------------------------------------------------
BATCH_SIZES = tuple(range(8, 49, 4))


def batch_lattice_sizes(count: int = 512, seed: int = 3) -> Dict[int, int]:
    """L -> number of lattices of that size."""
    import numpy as np
    rng = np.random.default_rng(seed)
    Ls = rng.choice(np.array(BATCH_SIZES), size=count)
    return {int(L): int((Ls == L).sum()) for L in BATCH_SIZES if (Ls == L).any()}


def batch_lattice_mcin(L: int, replicas: int = 16, steps: Tuple[int, int, int] = (1000, 10000, 1)) -> McInput:
    """The input of one lattice of the batch (its 16 temperatures)."""
    text = lattice_mcin(SC, L, [(1e-3, NN)], tem_range=(2.0, 25.0, replicas), tems_mode="log",
                        biquad=(1e-4, NN), dm=(2e-4, NN), pt=True, pt_steps_swap=10, steps=steps)
    return parse_mcin(text, seedname=f"batch_L{L}")
