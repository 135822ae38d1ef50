"""Writers of the reference's output files, byte-compatible in layout.

Formats follow ESpinS src/mcarlo.F90:106-200 (headers), :784-818 (rows) and
src/pt.F90:1040-1085:
* ``seed_mc.dat``       format 125: (f9.4,2x,6(E15.8,2x)) per temperature
* ``seed_pm.dat``       '#T=' line (1x,a,2x,f9.4), rows (2x,E15.8,10x,E15.8)
* ``seed_sconfig.dat``  date line, (3I6) supercell, (2I6) N and tems_num, then
                        per temperature (F12.6) T and (3F12.6) spins
* ``seed_binerror.dat`` '#T=' line, rows (2x,I8,8x,E15.8,3x,E15.8)
* ``seed.mcout``        the MONTECARLO summary block of mcarlo.F90:736-753 /
                        pt.F90:1000-1010 (format 124)
* ``seed_op.dat``, ``seed_staggered.dat``
                        headers of mcarlo.F90:144-162, rows format 126:
                        (3x,f9.4,5x,E15.8,6x,E15.8,7x,E15.8,5x) (:772-782)
* ``seed_spincorr.dat`` header of mcarlo.F90:131-141, rows
                        (f9.4,1x,I5,6x,a3,4x,i3,6x,a3,4x,i3,8x,f12.9,10x,f12.9,12x,f12.9)
                        per temperature, shell and species pair (:760-770)
* ``seed_energy-T###.dat`` one file per temperature (energy_write): date line,
                        '(3x,a,f9.4)' '# T = ', '(3x,i16)' the number of
                        measurements, then '(I14,4x,1E16.8)' measurement index
                        and running E/N (get_quant.F90:1130-1191)
* ``seed_sf-T###.dat``  structure factor per temperature: rows (3x,E15.8) x 3
                        (qpt_x, qpt_y, S) or x 5 with sfactor_polar (S, S - NSF,
                        NSF) in the plane coordinates of get_quant.F90:720-822
With the order parameter or the staggered magnetisation switched on, _pm.dat
gains the P(OP) / P(SM) columns and _binerror.dat their error columns
(mcarlo.F90:174-215 and :784-818, pt.F90:159-200 and :1050-1073).
"""
from __future__ import annotations

import datetime
import math
import os
from typing import Sequence

import numpy as np


def fortran_e(x: float, w: int = 15, d: int = 8) -> str:
    """Fortran Ew.d: 0.ddddddddE+xx, right-justified in w characters."""
    x = float(x)
    if x == 0.0 or not math.isfinite(x):
        if not math.isfinite(x):
            return ("NaN" if math.isnan(x) else ("-Infinity" if x < 0 else "Infinity")).rjust(w)
        body = "0." + "0" * d + "E+00"
        return body.rjust(w)
    sign = "-" if x < 0 else ""
    # the d significant digits of the exact binary value, correctly rounded
    mant, ex = f"{abs(x):.{d - 1}E}".split("E")
    digits = mant.replace(".", "")
    e = int(ex) + 1
    if abs(e) <= 99:
        s = f"{sign}0.{digits}E{'+' if e >= 0 else '-'}{abs(e):02d}"
    else:  # a three-digit exponent takes the place of the letter
        s = f"{sign}0.{digits}{'+' if e >= 0 else '-'}{abs(e):03d}"
    return s.rjust(w)


def fortran_f(x: float, w: int, d: int) -> str:
    s = f"{x:.{d}f}"
    if s.startswith("0.") and len(s) > w:
        s = s[1:]
    elif s.startswith("-0.") and len(s) > w:
        s = "-" + s[2:]
    return s.rjust(w) if len(s) <= w else "*" * w


def _date() -> str:
    now = datetime.datetime.now()
    return now.strftime("%d%b%Y").lstrip("0").rjust(9), now.strftime("%H:%M:%S")


def write_mc_dat(path: str, tems: Sequence[float], data: np.ndarray, n: int) -> None:
    """data: (R, 6) normalised <E>,<E2>,<E4>,<|m|>,<m2>,<m4> (mcarlo.F90:713-757)."""
    d, t = _date()
    with open(path, "w") as fh:
        fh.write(f" #written on {d} at {t} \n")
        fh.write(" #------------------------------------------------- MONTECARLO --------"
                 "-----------------------------------------#\n")
        fh.write(" # Temp      Magnetization     Energy_ave          C_M              Sus"
                 "              U_E              U_M       #\n")
        fh.write(" #-----------------------------------------------------------------------"
                 "---------------------------------------#\n")
        for T, row in zip(tems, data):
            for line in [mc_dat_row(T, row, n)]:
                fh.write(line + "\n")


def observables(T: float, row: np.ndarray, n: int):
    beta = 1.0 / T
    E, E2, E4, M, M2, M4 = row
    C = beta * beta * (E2 - E ** 2) / n
    chi = beta * (M2 - M ** 2) * n
    UE = 1.0 - (1.0 / 3.0) * (E4 / E2 ** 2)
    UM = 1.0 - (1.0 / 3.0) * (M4 / M2 ** 2)
    return M, E / n, C, chi, UE, UM


def mc_dat_row(T: float, row: np.ndarray, n: int) -> str:
    vals = observables(T, row, n)
    return fortran_f(T, 9, 4) + "".join("  " + fortran_e(v) for v in vals)


# Header lines of _pm.dat and _binerror.dat by (order parameter, staggered,
# parallel tempering): mcarlo.F90:174-215, pt.F90:159-200.
_PM_HEAD = {
    (True, True, False): [
        '#------------------------------------- MONTECARLO -------------------------------------------#',
        '#       M or OP                 P(M)                     P(OP)               P(Staggered_m)  #',
        '#--------------------------------------------------------------------------------------------#',
    ],
    (True, False, False): [
        '#-------------------------- MONTECARLO -------------------------------#',
        '#       M or OP                 P(M)                     P(OP)        #',
        '#---------------------------------------------------------------------#',
    ],
    (False, True, False): [
        '#-------------------------- MONTECARLO -----------------------------#',
        '# M or Staggered                P(M)                P(Staggered_m)  #',
        '#-------------------------------------------------------------------#',
    ],
    (False, False, False): [
        '#----------------- MONTECARLO -------------------#',
        '#        M                      P(M)             #',
        '#------------------------------------------------#',
    ],
    (True, True, True): [
        '#-------------------------------------- MONTECARLO ------------------------------------------#',
        '#       M or OP                 P(M)                     P(OP)               P(Staggered_m)  #',
        '#--------------------------------------------------------------------------------------------#',
    ],
    (True, False, True): [
        '#---------------------------- MONTECARLO -----------------------------#',
        '#       M or OP                 P(M)                     P(OP)        #',
        '#---------------------------------------------------------------------#',
    ],
    (False, True, True): [
        '#--------------------------- MONTECARLO-----------------------------#',
        '# M or Staggered                P(M)                P(Staggered_m)  #',
        '#-------------------------------------------------------------------#',
    ],
    (False, False, True): [
        '#----------------- MONTECARLO -------------------#',
        '#        M                      P(M)             #',
        '#------------------------------------------------#',
    ],
}

_BIN_HEAD = {
    (True, True, False): [
        '#------------------------------------ MONTECARLO ------------------------------------------#',
        '#  Binning_level     Error(E)          Error(M)        Error(OP)       Error(Staggered_m)  #',
        '#------------------------------------------------------ ------------------------------------#',
    ],
    (True, False, False): [
        '#------------------------- MONTECARLO -------------------------------#',
        '#  Binning_level     Error(E)          Error(M)         Error(OP)    #',
        '#--------------------------------------------------------------------#',
    ],
    (False, True, False): [
        '#----------------------------- MONTECARLO -------------------------------#',
        '#  Binning_level     Error(E)          Error(M)      Error(Staggered_m)  #',
        '#------------------------------------------------------------------------#',
    ],
    (False, False, False): [
        '#------------------- MONTECARLO -----------------#',
        '#  Block_length      Error(E)          Error(M)  #',
        '#------------------------------------------------#',
    ],
    (True, True, True): [
        '#------------------------------------- MONTECARLO -----------------------------------------#',
        '#  Binning_level     Error(E)          Error(M)        Error(OP)       Error(Staggered_m)  #',
        '#------------------------------------------------------------------------------------------#',
    ],
    (True, False, True): [
        '#--------------------------- MONTECARLO -----------------------------#',
        '#  Binning_level     Error(E)          Error(M)         Error(OP)    #',
        '#--------------------------------------------------------------------#',
    ],
    (False, True, True): [
        '#----------------------------- MONTECARLO -------------------------------#',
        '#  Binning_level     Error(E)          Error(M)      Error(Staggered_m)  #',
        '#------------------------------------------------------------------------#',
    ],
    (False, False, True): [
        '#------------------- MONTECARLO -----------------#',
        '#  Block_length      Error(E)          Error(M)  #',
        '#------------------------------------------------#',
    ],
}


def write_pm_dat(path: str, tems, pm: np.ndarray, m_min: float, m_max: float, pm_op=None, pm_sm=None,
                 pt: bool = False) -> None:
    """pm: (R, nf) P(M); pm_op / pm_sm: (R, nf) P(OP) / P(SM) columns or None."""
    nf = pm.shape[1]
    dm = (m_max - m_min) / (nf - 1)
    m_array = [m_min + i * dm for i in range(nf)]
    cols = [c for c in (pm_op, pm_sm) if c is not None]
    d, t = _date()
    with open(path, "w") as fh:
        fh.write(f" #written on {d} at {t} \n")
        for ln in _PM_HEAD[(pm_op is not None, pm_sm is not None, bool(pt))]:
            fh.write(" " + ln + "\n")
        for k, (T, row) in enumerate(zip(tems, pm)):
            fh.write(" #T=  " + fortran_f(T, 9, 4) + "\n")
            for f, (m, p) in enumerate(zip(m_array, row)):
                fh.write("  " + fortran_e(m) + " " * 10 + fortran_e(p)
                         + "".join(" " * 10 + fortran_e(c[k][f]) for c in cols) + "\n")


def obs_row(T: float, row3, n: int) -> str:
    """Format 126 row of _op.dat / _staggered.dat from <|x|>, <x^2>, <x^4>
    (x = OP or SM): T, <|x|>, beta (<x^2> - <|x|>^2) N, 1 - <x^4> / (3 <x^2>^2)."""
    beta = 1.0 / T
    a, a2, a4 = row3
    sus = beta * (a2 - a ** 2) * n
    U = 1.0 - (1.0 / 3.0) * (a4 / a2 ** 2)
    return format126(T, a, sus, U)


def format126(T: float, v1: float, v2: float, v3: float) -> str:
    """mcarlo.F90 format 126: (3x,f9.4,5x,E15.8,6x,E15.8,7x,E15.8,5x); the
    trailing 5x writes nothing (position editing at the end of a record)."""
    return ("   " + fortran_f(T, 9, 4) + " " * 5 + fortran_e(v1) + " " * 6 + fortran_e(v2)
            + " " * 7 + fortran_e(v3))


def write_obs_dat(path: str, kind: str, tems, obs_data: np.ndarray, n: int) -> None:
    """kind 'op' (_op.dat, obs_data[:, 0:3]) or 'staggered' (_staggered.dat, [:, 3:6])."""
    d, t = _date()
    if kind == "op":
        head = [" #------------------------------- MONTECARLO -----------------------------------#",
                " #    Temp              OP                 Sus_OP                 U_OP          #",
                " #------------------------------------------------------------------------------#"]
        c0 = 0
    else:
        head = [" #------------------------------- MONTECARLO --------------------------------#",
                " #    Temp         Staggered_m          Sus_Staggered_m       U_Staggered_m  #",
                " #---------------------------------------------------------------------------#"]
        c0 = 3
    with open(path, "w") as fh:
        fh.write(f" #written on {d} at {t} \n")
        for ln in head:
            fh.write(ln + "\n")
        for T, row in zip(tems, obs_data):
            fh.write(obs_row(T, row[c0:c0 + 3], n) + "\n")


def write_sconfig(path: str, supercell, tems, spins: np.ndarray) -> None:
    """spins: (R, N, 3) as the reference's global_spin_matrix(3,N,R)."""
    d, t = _date()
    R, N, _ = spins.shape
    with open(path, "w") as fh:
        fh.write(f" Created on {d} at {t} \n")
        fh.write("".join(f"{int(v):6d}" for v in supercell) + "\n")
        fh.write(f"{N:6d}{R:6d}\n")
        for T, blk in zip(tems, spins):
            fh.write(fortran_f(T, 12, 6) + "\n")
            for s in blk:
                fh.write("".join(fortran_f(v, 12, 6) for v in s) + "\n")


def read_sconfig(path: str, n: int, tems) -> np.ndarray:
    """``mcarlo_read_sconfig`` (get_quant.F90:543-598): spins normalised to unit length."""
    with open(path) as fh:
        lines = fh.read().splitlines()
    nw, nt = (int(x) for x in lines[2].split())
    if nw != n:
        raise ValueError("Wrong matrix size in mcarlo: read_sconfig")
    if nt != len(tems):
        raise ValueError("Wrong temperature number in mcarlo: read_sconfig")
    out = np.zeros((nt, n, 3))
    pos = 3
    for k in range(nt):
        tt = float(lines[pos]); pos += 1
        if abs(tt - tems[k]) > 1e-4:
            raise ValueError("Mismatch in temperatures: read_sconfig")
        blk = np.array([[float(v) for v in lines[pos + j].split()[:3]] for j in range(n)])
        pos += n
        if np.any(np.all(np.abs(blk) < 1e-4, axis=1)):
            raise ValueError("All components of an spin in block are zero")
        out[k] = blk / np.sqrt((blk * blk).sum(axis=1, keepdims=True))
    return out


def spincorr_row(T: float, shell: int, sym1: str, t1: int, sym2: str, t2: int, v1: float, v2: float,
                 v3: float) -> str:
    """(f9.4,1x,I5,6x,a3,4x,i3,6x,a3,4x,i3,8x,f12.9,10x,f12.9,12x,f12.9)."""
    def a3(x):
        return (x + "   ")[:3]
    return (fortran_f(T, 9, 4) + " " + f"{shell:5d}" + " " * 6 + a3(sym1) + " " * 4 + f"{t1:3d}" + " " * 6
            + a3(sym2) + " " * 4 + f"{t2:3d}" + " " * 8 + fortran_f(v1, 12, 9) + " " * 10 + fortran_f(v2, 12, 9)
            + " " * 12 + fortran_f(v3, 12, 9))


def write_spincorr(path: str, tems, sc: np.ndarray, sc_abs: np.ndarray, sc_tot: np.ndarray, symbols) -> None:
    """sc, sc_abs, sc_tot: (R, shells, species, species), normalised.  The
    species symbols print with a capital first letter (param_uppercase,
    parameters.F90:1047-1070)."""
    symbols = [x[:1].upper() + x[1:] for x in symbols]
    d, t = _date()
    with open(path, "w") as fh:
        fh.write(f" #written on {d} at {t} \n")
        fh.write(" #---------------------------------------------------- MONTECARLO "
                 "----------------------------------------------------#\n")
        fh.write(" #  Temp    Shell   Atom1   Type1   Atom2   Type2   "
                 "<\\sum_{ij} Si.Sj/N>   <\\sum_{ij}|Si.Sj|/N>   <|\\sum_{ij}Si.Sj|/N> #\n")
        fh.write(" #----------------------------------------------------------------"
                 "----------------------------------------------------#\n")
        for k, T in enumerate(tems):
            S, nsp = sc.shape[1], sc.shape[2]
            for l in range(S):
                for a in range(nsp):
                    for b in range(nsp):
                        fh.write(spincorr_row(T, l + 1, symbols[a], a + 1, symbols[b], b + 1, sc[k, l, a, b],
                                              sc_abs[k, l, a, b], sc_tot[k, l, a, b]) + "\n")


def energy_series_name(seedname: str, n: int) -> str:
    """seed_energy-T###.dat of the n-th temperature (1-based, three digits)."""
    return f"{seedname}_energy-T{n // 100 % 10}{n // 10 % 10}{n % 10}.dat"


class EnergySeries:
    """The energy series files of open_E_unit / write_E / close_E_unit: rows
    are appended in measurement order as the run produces them."""

    def __init__(self, base: str, tems, nsteps: int, n: int):
        self.n = n
        self.count = 0
        d, t = _date()
        folder, seed = os.path.split(base)
        self.fh = []
        for k, T in enumerate(tems, start=1):
            fh = open(os.path.join(folder, energy_series_name(seed, k)), "w")
            fh.write(f" #written on {d} at {t} \n")
            fh.write("   # T = " + fortran_f(T, 9, 4) + "\n")
            fh.write("   " + f"{int(nsteps):16d}" + "\n")
            self.fh.append(fh)

    def append(self, energies: np.ndarray) -> None:
        """energies: (measurements, R) running energies, oldest first."""
        m = energies.shape[0]
        for t, fh in enumerate(self.fh):
            fh.write("".join(f"{self.count + i + 1:14d}    " + fortran_e(energies[i, t] / self.n, 16, 8) + "\n"
                             for i in range(m)))
        self.count += m

    def close(self) -> None:
        for fh in self.fh:
            fh.close()
        self.fh = []


def sfactor_plane_coords(corner, q1v, q2v, mesh):
    """(qpt_x, qpt_y) of every q-point in loop_xy order, in the orthogonal
    frame of the (q1, q2) plane (mcarlo_structure_factor_write_mc,
    get_quant.F90:745-813)."""
    from .mcin import _recip_lattice
    q1v, q2v, corner = (np.asarray(v, dtype=float) for v in (q1v, q2v, corner))
    z = np.cross(q1v, q2v)
    y = np.cross(z, q1v)
    q1mod, q2mod, ymod = (math.sqrt(float(v @ v)) for v in (q1v, q2v, y))
    qvec = np.array([q1v, q2v, z / math.sqrt(float(z @ z))])
    avec, _ = _recip_lattice(qvec)
    cosyq2 = float(y @ q2v) / (ymod * q2mod)
    cosq1q2 = float(q1v @ q2v) / (q1mod * q2mod)
    m1, m2 = mesh
    out = []
    for xy in range((m1 + 1) * (m2 + 1)):
        lx, ly = xy // (m2 + 1), xy % (m2 + 1)
        a = lx / float(m1) + float(corner @ avec[0]) / (2.0 * math.pi)
        b = ly / float(m2) + float(corner @ avec[1]) / (2.0 * math.pi)
        out.append((a * q1mod + b * q2mod * cosq1q2, b * q2mod * cosyq2))
    return out


def write_sfactor(base: str, tems, sf: np.ndarray, coords, polar: bool) -> None:
    """One seed_sf-T###.dat per temperature; sf (R, nq, 3) normalised."""
    folder, seed = os.path.split(base)
    for k, _ in enumerate(tems, start=1):
        name = os.path.join(folder, f"{seed}_sf-T{k // 100 % 10}{k // 10 % 10}{k % 10}.dat")
        with open(name, "w") as fh:
            for (x, y), v in zip(coords, sf[k - 1]):
                vals = [x, y] + (list(v) if polar else [v[0]])
                fh.write("".join("   " + fortran_e(u) for u in vals) + "\n")


def write_binerror(path: str, tems, binning: np.ndarray, levels, n: int, pt: bool, obs_binning=None,
                   op: bool = False, sm: bool = False) -> None:
    """binning: (R, nlev, 2) E/N and |m| rows; obs_binning: (R, nlev, 2) |OP|
    and SM rows, of which the op / sm ones are written."""
    ncol = 2 + int(op) + int(sm)
    with open(path, "w") as fh:
        for ln in _BIN_HEAD[(op, sm, bool(pt))]:
            fh.write(" " + ln + "\n")
        for k, (T, b) in enumerate(zip(tems, binning)):
            fh.write(" #T=  " + (fortran_f(T, 6, 2) if pt else fortran_f(T, 9, 4)) + "\n")
            for l, (lv, row) in enumerate(zip(levels, b)):
                row = list(row)
                if op:
                    row.append(obs_binning[k][l][0])
                if sm:
                    row.append(obs_binning[k][l][1])
                row = np.asarray(row)
                vals = np.sqrt(np.maximum(row, 0.0)) if pt else np.sqrt(np.maximum(row / n, 0.0))
                # mcarlo.F90 writes the level as I3 when both extra rows are on
                lvs = f"{int(lv):3d}" if (ncol == 4 and not pt) else f"{int(lv):8d}"
                fh.write(f"  {lvs}        " + "   ".join(fortran_e(v) for v in vals[:ncol]) + "\n")


def _steps_line(T: float, tot: int, rej: int, tag: str, pt: bool) -> str:
    """Format 124 of mcarlo.F90:853 (f10.8, 1x, a) / pt.F90:1126 (f10.8, 4x, a)."""
    ratio = (tot - rej) / tot if tot else 0.0
    return (f"   {fortran_f(T, 9, 4)} {tot:14d} {rej:14d}     {tot - rej:14d}       {ratio:10.8f}"
            + (" " * 4 if pt else " ") + "  <-- " + tag)


def mcout_block(tems, res: dict, n: int, pt: bool) -> str:
    """The .mcout summary of the measurement phase, line for line as the
    reference prints it.

    mcarlo (mcarlo.F90:736-753): per temperature the WARMUP and MCARLO lines
    (format 124; ' No Warm-up step is done! ' without warm-up), the energy
    triple, Delta E and Delta M, a dashed line.  pt_mcarlo (pt.F90:983-1021):
    the final swap table (format 128; Fortran writes no trailing blanks for a
    closing 2x) and then per temperature the MCARLO line, the energy triple
    marked ENERGY3, Delta E, Delta M and the dashed line.  The sections that
    pt_mcarlo prints during its warm-up (WARMUP1, WARMUP2, the swap log) are
    not part of this block."""
    out = []
    norm = 1.0 / res["steps_mc_eff"]
    mark = "  <-- ENERGY3" if pt else "  <-- ENERGY"
    if pt:
        out += ["", " *----------------------------------- MONTECARLO ------------------------------------*",
                " |  Temp_i     Temp_f         Tot-Swaps       Rej-Swaps      Acc-Swaps  Acc/Tot Ratio|",
                " +-----------------------------------------------------------------------------------+"]
        for t, T in enumerate(tems):
            tries, acc = (int(x) for x in res["num_swaps"][t])
            Tf = tems[int(res["map"][t]) - 1]
            ratio = acc / tries if tries else 0.0
            out.append(f"  {fortran_f(T, 9, 4)}  {fortran_f(Tf, 9, 4)} {tries:14d} {tries - acc:14d} "
                       f"{acc:14d}   {ratio:14.8f}")
        out += ["", " *----------------------------------- MONTECARLO ------------------------------------*",
                " |     Temp      Total Steps    Rejected Steps    Accepted Steps   Acc/Tot Ratio     |",
                " +-----------------------------------------------------------------------------------+"]
    for t, T in enumerate(tems):
        if not pt:
            if int(res["steps_tot"][0]) > 0:
                out.append(_steps_line(T, int(res["steps_tot"][0]), int(res["rejected"][t][0]), "WARMUP", False))
            else:
                out.append("  No Warm-up step is done! ")
        out.append(_steps_line(T, int(res["steps_tot"][1]), int(res["rejected"][t][1]), "MCARLO", pt))
        E = res["energy"][t]
        out.append(f"     Initial Energy                           = {fortran_e(E[0], 15, 7)}{mark}")
        out.append(f"     Final Energy by adding differences       = {fortran_e(E[1], 15, 7)}{mark}")
        out.append(f"     Final Energy by direct calculations      = {fortran_e(E[2], 15, 7)}{mark}")
        d = res["data"][t]
        dE = math.sqrt(max(d[1] - d[0] ** 2, 0.0) * norm) / n
        dM = math.sqrt(max(d[4] - d[3] ** 2, 0.0) * norm)
        out.append(f"                                 Delta E      = +/- {dE:15.9f}")
        out.append(f"                                 Delta M      = +/- {dM:15.9f}")
        out.append(" " + "-" * 85)
    return "\n".join(out) + "\n"