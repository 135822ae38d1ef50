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

Run from the repository root:  python tests/golden/make_golden.py [reference_dir]
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
            gold.update(parse_mcout(fh.read()))
        mcdat = os.path.join(base, seed + "_mc.dat")
        if os.path.exists(mcdat):
            with open(mcdat) as fh:
                gold["mc_dat"] = parse_mc_dat(fh.read())
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
                gold["pm_dat"] = parse_pm_dat(fh.read(), PM_TEMPS[name])
        scf = os.path.join(base, seed + "_sconfig.dat")
        if keep != 0 and os.path.exists(scf):
            with open(scf) as fh:
                sc, temps, spins = parse_sconfig(fh.read(), keep)
            np.savez_compressed(os.path.join(HERE, name + "_sconfig.npz"),
                                supercell=np.array(sc), temps=temps, spins=spins)
        with open(os.path.join(HERE, name + "_golden.json"), "w") as fh:
            json.dump(gold, fh, indent=1)
        print(name, len(gold["rows"]), "rows", len(gold.get("seeds", [])), "seeds")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
