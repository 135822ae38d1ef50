"""Extract the golden fixtures used by the tests from the reference's examples.

The reference (ESpinS) ships no unit tests; its only known answers are the
example runs under ``examples/example0*/reference/``.  This script reads those
outputs as text and writes small fixtures next to itself:

* ``<name>.mcin``                       the example's Monte Carlo input
* ``<name>_golden.json``                seeds, per-temperature accept/reject
                                        counts and the energy triple of the
                                        ``.mcout`` (mcarlo.F90:736-753 format),
                                        and the ``_mc.dat`` rows; the
                                        ``_op.dat`` / ``_staggered.dat`` rows
                                        when the example wrote them; the
                                        ``_pm.dat`` columns of the temperatures
                                        listed in PM_TEMPS; the _spincorr.dat
                                        rows of the temperatures in SC_TEMPS
* ``<name>_sconfig.npz``                final spins per temperature
                                        (``_sconfig.dat``, 6 decimals)

For the byte-compatibility tests of the output writers the fixture also keeps
verbatim text: every ``_mc.dat`` data line, the ``.mcout`` summary block of
the first temperatures (with parallel tempering also the final swap table and
its numbers), the header and first temperature block of ``_sconfig.dat`` and
the header and kept blocks of ``_pm.dat``.

Run from the repository root, naming the checkout of the reference:
    python tests/golden/make_golden.py <reference_dir>
"""
from __future__ import annotations

import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

EXAMPLES = {
    # name: (directory, seedname, max temperatures kept in the sconfig fixture)
    "ex01_cubic": ("examples/example01/reference", "cubic", None),
    "ex03_fef3": ("examples/example03/reference", "fef3", None),
    "ex05_snwo": ("examples/example05/reference", "snwo", None),
    "ex02_cubic_pt": ("examples/example02/reference", "cubic", 4),
    "ex04_bmno_mc": ("examples/example04/reference/mc_with_uniform_temperatures", "bmno", 0),
}

# temperatures whose _pm.dat block is kept (the ones the seed-exact replays reach)
PM_TEMPS = {"ex03_fef3": [11.1111], "ex01_cubic": [], "ex05_snwo": [], "ex02_cubic_pt": [], "ex04_bmno_mc": []}

# temperatures whose _spincorr.dat rows are kept
SC_TEMPS = {"ex05_snwo": [4.0]}


def parse_spincorr(text: str, keep):
    """Rows (T, shell, type1, type2, sum, sum_abs, tot_abs) at the kept temperatures."""
    rows, lines = [], []
    for ln in text.splitlines():
        s = ln.split()
        if not s or s[0].startswith("#"):
            continue
        t = float(s[0])
        if any(abs(t - k) < 1e-4 for k in keep):
            rows.append([t, int(s[1]), int(s[3]), int(s[5])] + [float(x) for x in s[6:9]])
            lines.append(ln)
    return rows, lines


def parse_pm_dat(text: str, keep):
    """{T: rows} of a _pm.dat file for the temperatures in keep."""
    out, cur = {}, None
    for ln in text.splitlines():
        s = ln.strip()
        if s.startswith("#T="):
            t = float(s[3:])
            cur = [] if any(abs(t - k) < 1e-4 for k in keep) else None
            if cur is not None:
                out["%.4f" % t] = cur
            continue
        if not s or s.startswith("#") or cur is None:
            continue
        cur.append([float(x) for x in s.split()])
    return out


def pm_dat_lines(text: str, keep):
    """{T: verbatim lines} of the kept _pm.dat blocks, '#T=' line first."""
    out, cur = {}, None
    for ln in text.splitlines():
        s = ln.strip()
        if s.startswith("#T="):
            t = float(s[3:])
            cur = [ln] if any(abs(t - k) < 1e-4 for k in keep) else None
            if cur is not None:
                out["%.4f" % t] = cur
            continue
        if cur is not None and s and not s.startswith("#"):
            cur.append(ln)
    return out


def parse_mcout(text: str) -> dict:
    out = {"seeds": [], "rows": []}
    lines = text.splitlines()
    for i, ln in enumerate(lines):
        if "Seeds:" in ln:
            j = i + 1
            while j < len(lines) and not lines[j].strip().startswith("*"):
                out["seeds"] += [int(x) for x in re.findall(r"-?\d+", lines[j])]
                j += 1
    cur = None
    for ln in lines:
        m = re.match(r"\s+([\d.]+)\s+(\d+)\s+(\d+)\s+(\d+)\s+([\d.]+)\s+<-- (WARMUP|MCARLO)$", ln)
        if m:
            t = float(m.group(1))
            if m.group(6) == "WARMUP" or cur is None or cur.get("T") != t:
                cur = {"T": t}
                out["rows"].append(cur)
            key = "warmup" if m.group(6) == "WARMUP" else "mc"
            cur[key] = [int(m.group(2)), int(m.group(3))]
            continue
        m = re.match(r"\s+(Initial Energy|Final Energy by adding differences|Final Energy by direct calculations)"
                     r"\s+=\s+(\S+)\s+<-- ENERGY(\d?)", ln)
        if m and cur is not None:
            k = {"Initial Energy": "E_init", "Final Energy by adding differences": "E_add",
                 "Final Energy by direct calculations": "E_direct"}[m.group(1)]
            cur[k] = float(m.group(2))
            continue
        m = re.match(r"\s+Delta ([EM])\s+=\s+\+/-\s+(\S+)", ln)
        if m and cur is not None:
            cur["d" + m.group(1)] = float(m.group(2))
    return out


MCOUT_BLOCK_TEMPS = 4


def mcout_blocks(text: str, pt: bool):
    """Verbatim lines of the .mcout summary: per temperature the block from its
    first '<-- WARMUP' / '<-- MCARLO' line of the measurement summary to the
    dashed line after 'Delta M' (mcarlo.F90:736-753, pt.F90:1011-1021), for the
    first MCOUT_BLOCK_TEMPS temperatures; with pt also the final swap table
    (pt.F90:983-990): its three header lines and rows."""
    lines = text.splitlines()
    out = {"blocks": [], "swap_lines": []}
    if pt:
        # the last MONTECARLO swap table
        idx = [i for i, ln in enumerate(lines) if "Temp_i     Temp_f" in ln]
        if idx:
            i = idx[-1] - 1
            j = i + 3
            while j < len(lines) and lines[j].strip():
                j += 1
            out["swap_lines"] = lines[i:j]
    i = 0
    while i < len(lines) and len(out["blocks"]) < MCOUT_BLOCK_TEMPS:
        ln = lines[i]
        starts = ln.rstrip().endswith("<-- WARMUP") or (ln.rstrip().endswith("<-- MCARLO") and not (
            i > 0 and lines[i - 1].rstrip().endswith("<-- WARMUP")))
        # the measurement summary lines of PT are marked ENERGY3
        if starts and (not pt or (i + 1 < len(lines) and "ENERGY3" in lines[i + 1])):
            j = i
            while j < len(lines) and not lines[j].startswith(" ----"):
                j += 1
            out["blocks"].append(lines[i:j + 1])
            i = j + 1
            continue
        i += 1
    return out


def parse_swaps(lines):
    """(T_i, T_f, tries, rejected, accepted, ratio) rows of a swap table."""
    rows = []
    for ln in lines:
        s = ln.split()
        if len(s) == 6 and not ln.strip().startswith(("|", "*", "+")):
            rows.append([float(s[0]), float(s[1]), int(s[2]), int(s[3]), int(s[4]), float(s[5])])
    return rows


def parse_mc_dat(text: str):
    rows = []
    for ln in text.splitlines():
        s = ln.strip()
        if not s or s.startswith("#"):
            continue
        rows.append([float(x) for x in s.split()])
    return rows


def parse_sconfig(text: str, keep):
    lines = text.splitlines()
    sc = [int(x) for x in lines[1].split()]
    nw, nt = (int(x) for x in lines[2].split())
    temps, spins = [], []
    pos = 3
    nkeep = nt if keep is None else min(nt, keep)
    for t in range(nkeep):
        temps.append(float(lines[pos])); pos += 1
        spins.append([[float(v) for v in lines[pos + j].split()] for j in range(nw)])
        pos += nw
    return sc, np.array(temps), np.array(spins)


def main(ref_root: str) -> None:
    for name, (d, seed, keep) in EXAMPLES.items():
        base = os.path.join(ref_root, d)
        with open(os.path.join(base, seed + ".mcin")) as fh:
            mcin = fh.read()
        with open(os.path.join(HERE, name + ".mcin"), "w") as fh:
            fh.write(mcin)
        gold = {"source": os.path.join(d, seed)}
        with open(os.path.join(base, seed + ".mcout")) as fh:
            mcout = fh.read()
        gold.update(parse_mcout(mcout))
        pt = bool(re.search(r"^\s*pt\s*=\s*\.true\.", mcin, re.I | re.M))
        blk = mcout_blocks(mcout, pt)
        gold["mcout_blocks"] = blk["blocks"]
        if pt:
            gold["swap_lines"] = blk["swap_lines"]
            gold["swaps"] = parse_swaps(blk["swap_lines"])
        mcdat = os.path.join(base, seed + "_mc.dat")
        if os.path.exists(mcdat):
            with open(mcdat) as fh:
                text = fh.read()
            gold["mc_dat"] = parse_mc_dat(text)
            gold["mc_dat_lines"] = [ln for ln in text.splitlines() if ln.strip() and not ln.strip().startswith("#")]
            gold["mc_dat_head"] = text.splitlines()[1:4]
        for kind in ("op", "staggered"):
            f = os.path.join(base, seed + "_" + kind + ".dat")
            if os.path.exists(f):
                with open(f) as fh:
                    text = fh.read()
                gold[kind + "_dat"] = parse_mc_dat(text)
                # a few rows verbatim, for the writer's format check
                gold[kind + "_dat_lines"] = [ln for ln in text.splitlines() if ln.strip()
                                             and not ln.strip().startswith("#")][:3]
        scf_ = os.path.join(base, seed + "_spincorr.dat")
        if SC_TEMPS.get(name) and os.path.exists(scf_):
            with open(scf_) as fh:
                gold["spincorr_dat"], gold["spincorr_dat_lines"] = parse_spincorr(fh.read(), SC_TEMPS[name])
        pmf = os.path.join(base, seed + "_pm.dat")
        if PM_TEMPS.get(name) and os.path.exists(pmf):
            with open(pmf) as fh:
                text = fh.read()
            gold["pm_dat"] = parse_pm_dat(text, PM_TEMPS[name])
            gold["pm_dat_head"] = text.splitlines()[1:4]
            gold["pm_dat_lines"] = pm_dat_lines(text, PM_TEMPS[name])
        scf = os.path.join(base, seed + "_sconfig.dat")
        if keep != 0 and os.path.exists(scf):
            with open(scf) as fh:
                text = fh.read()
            sc, temps, spins = parse_sconfig(text, keep)
            nw = int(text.splitlines()[2].split()[0])
            # header after the date line, and the first temperature's block
            # (small lattices only)
            if nw <= 256:
                gold["sconfig_lines"] = text.splitlines()[1:3 + 1 + nw]
            np.savez_compressed(os.path.join(HERE, name + "_sconfig.npz"),
                                supercell=np.array(sc), temps=temps, spins=spins)
        with open(os.path.join(HERE, name + "_golden.json"), "w") as fh:
            json.dump(gold, fh, indent=1)
        print(name, len(gold["rows"]), "rows", len(gold.get("seeds", [])), "seeds")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <reference_dir>")
    main(sys.argv[1])
