"""Reader for ESpinS ``.mcin`` input files (the keywords the Monte Carlo path uses).

Follows the reference's keyword semantics (ESpinS ``src/parameters.F90``):

* the file is lower-cased, ``!`` and ``#`` start comments and blank lines are
  dropped (``param_in_file``, parameters.F90:1724-1805);
* a keyword matches a line that starts with it and is followed by ``=``, ``:``
  or a blank (``param_get_keyword``, parameters.F90:1808-1873); a keyword given
  twice is an error, as is any line left unconsumed at the end
  (parameters.F90:997-1030);
* logicals are true when the value contains ``t`` and false when it contains
  ``f`` (parameters.F90:1857-1864);
* ``begin X`` / ``end X`` blocks may carry a units line (``ang``/``bohr``, and
  ``ev``/``ryd`` for parameter blocks) (parameters.F90:2558-2846, 3061-3280).

Energies are converted to Kelvin exactly where the reference converts them:
exchange, biquadratic and DM in the table builders (jij.F90:163, bij.F90:126,
dij.F90:126), single-ion at parameters.F90:958 and the Zeeman field
(Tesla * mu_B / k_B) at parameters.F90:994.

Errors raise :class:`McinError`, the analogue of ``io_error``.
"""
from __future__ import annotations

import math
import re
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple

import numpy as np

# mc_constants (src/constants.F90:26-48)
PI = 3.141592653589793238462643383279
TWOPI = 2.0 * PI
BOHR = 0.5291772108
HART = 27.21138602
K_B = 8.6173303e-5          # eV/K
BOHR_MAGN = 5.7883818012e-5  # eV/T
EPS4 = 1.0e-4
EPS5 = 1.0e-5
EPS8 = 1.0e-8


class McinError(RuntimeError):
    """Input error; the reference stops through ``io_error`` in these cases."""


def _fnum(tok: str) -> float:
    """Fortran list-directed real: accepts d/D exponents."""
    t = tok.strip().replace("d", "e").replace("D", "e")
    try:
        return float(t)
    except ValueError as exc:
        raise McinError(f"Problem reading number '{tok}'") from exc


def _fint(tok: str) -> int:
    try:
        return int(tok.strip())
    except ValueError as exc:
        raise McinError(f"Problem reading integer '{tok}'") from exc


def _tokens(s: str) -> List[str]:
    return [t for t in re.split(r"[\s,]+", s.strip()) if t]


def _strip_all(s: str) -> str:
    return "".join(s.split())


@dataclass
class PairBlock:
    """Rows of a Jij/Bij/Dij_parameters block: fractional sites and value (eV)."""
    f1: np.ndarray      # (n, 3)
    f2: np.ndarray      # (n, 3)
    value: np.ndarray   # (n,)
    shell: Optional[np.ndarray] = None
    sigma: Optional[np.ndarray] = None


@dataclass
class McInput:
    seedname: str = ""
    # lattice
    real_lattice: np.ndarray = field(default_factory=lambda: np.eye(3))
    recip_lattice: np.ndarray = field(default_factory=lambda: np.eye(3))
    cell_volume: float = 1.0
    num_atoms: int = 0
    num_species: int = 0
    atoms_label: List[str] = field(default_factory=list)      # per species
    atoms_symbol: List[str] = field(default_factory=list)     # per species
    atoms_species_num: List[int] = field(default_factory=list)
    atoms_frac: np.ndarray = field(default_factory=lambda: np.zeros((0, 3)))  # species-major (num_atoms, 3)
    atoms_cart: np.ndarray = field(default_factory=lambda: np.zeros((0, 3)))
    mag_cell: np.ndarray = field(default_factory=lambda: np.zeros(0))          # species-major moments
    atom_species: List[int] = field(default_factory=list)     # species index per atom (0-based)
    supercell_size: Tuple[int, int, int] = (4, 4, 4)
    boundary_open: bool = False
    # temperatures / schedule
    tems_mode: str = "lin"
    tem_start: float = 5.0
    tem_end: float = 5.0
    tems_num: int = 1
    tems: np.ndarray = field(default_factory=lambda: np.array([5.0]))
    steps_warmup: int = 100000
    steps_mc: int = 200000
    steps_measure: int = 2
    initial_sconfig: str = "ferro"
    mcarlo_mode: str = "random"
    tilt_angles_max: float = 0.125
    seeds: Optional[List[int]] = None
    pt: bool = False
    pt_steps_swap: int = 1
    pt_print_swap: int = 10000
    # measurements
    lbinerror: bool = False
    binning_level: List[int] = field(default_factory=lambda: [1, 2, 3, 4, 5])
    lspincorr: bool = False
    lorderparam: bool = False
    lstaggered: bool = False
    staggered_coeff: Optional[np.ndarray] = None
    orderparam_axes_cart: Optional[np.ndarray] = None
    energy_write: bool = False
    energy_num_print: int = 1000
    lsfactor: bool = False
    lsfactor_polar: bool = False
    sfactor_polar: Optional[np.ndarray] = None      # cartesian (1/length)
    sfactor_corner: Optional[np.ndarray] = None
    sfactor_q1: Optional[np.ndarray] = None
    sfactor_q2: Optional[np.ndarray] = None
    sfactor_steps_measure: int = 100
    sfactor_2dqmesh: Optional[list] = None
    spin_glass: bool = False
    # Hamiltonian
    have_biquad: bool = False
    have_dm: bool = False
    have_singleion: bool = False
    have_field: bool = False
    jij: Optional[PairBlock] = None
    bij: Optional[PairBlock] = None
    dij: Optional[PairBlock] = None
    dij_vectors_cart: Optional[np.ndarray] = None   # (n, 3) unit vectors
    singleion_axes_cart: Optional[np.ndarray] = None  # (num_atoms, 3)
    singleion_parameters: Optional[np.ndarray] = None  # K
    field_axes_cart: Optional[np.ndarray] = None
    field_parameters: Optional[np.ndarray] = None      # K

    @property
    def num_supercell(self) -> int:
        a, b, c = self.supercell_size
        return a * b * c

    @property
    def num_total_atoms(self) -> int:
        return self.num_supercell * self.num_atoms


class _Lines:
    """The lower-cased, comment-stripped lines (``in_data``)."""

    def __init__(self, text: str):
        self.data: List[str] = []
        for raw in text.splitlines():
            d = raw.lower().lstrip()
            if not d or d[0] in "!#":
                continue
            i1, i2 = d.find("!"), d.find("#")
            cut = [i for i in (i1, i2) if i >= 0]
            if cut:
                d = d[: min(cut)]
            if d.strip():
                self.data.append(d.rstrip())

    # -- scalar keywords ---------------------------------------------------
    def keyword(self, key: str) -> Optional[str]:
        value = None
        for i, line in enumerate(self.data):
            if not line.startswith(key):
                continue
            nxt = line[len(key): len(key) + 1]
            if nxt not in ("=", ":", " ", ""):
                continue
            if value is not None:
                raise McinError(f"Found keyword {key} more than once in input file")
            v = line[len(key):].lstrip()
            if v[:1] in ("=", ":"):
                v = v[1:].lstrip()
            value = v
            self.data[i] = ""
        return value

    def logical(self, key: str, default: bool) -> bool:
        v = self.keyword(key)
        if v is None:
            return default
        if "t" in v:
            return True
        if "f" in v:
            return False
        raise McinError(f"Problem reading logical keyword {key}")

    def integer(self, key: str, default: int) -> int:
        v = self.keyword(key)
        if v is None:
            return default
        toks = _tokens(v)
        if not toks:
            raise McinError(f"Problem reading keyword {key}")
        return _fint(toks[0])

    def real(self, key: str, default: float) -> float:
        v = self.keyword(key)
        if v is None:
            return default
        toks = _tokens(v)
        if not toks:
            raise McinError(f"Problem reading keyword {key}")
        return _fnum(toks[0])

    def vector(self, key: str, length: int, conv) -> Optional[list]:
        v = self.keyword(key)
        if v is None:
            return None
        toks = _tokens(v)
        if len(toks) < length:
            raise McinError(f"Problem reading keyword {key}")
        return [conv(t) for t in toks[:length]]

    def range_vector(self, key: str) -> Optional[List[int]]:
        """``param_get_range_vector`` (parameters.F90:2245-2341): 1,3,5-8 or 4:10."""
        v = self.keyword(key)
        if v is None:
            return None
        if not v.strip():
            raise McinError(f"keyword {key} is blank")
        out: List[int] = []
        for part in re.split(r"[\s,;]+", v.strip()):
            if not part:
                continue
            m = re.fullmatch(r"(-?\d+)\s*[-:]\s*(\d+)", part)
            if m:
                a, b = int(m.group(1)), int(m.group(2))
                out.extend(range(min(a, b), max(a, b) + 1))
            else:
                out.append(_fint(part))
        if len(set(out)) != len(out):
            raise McinError(f"Error parsing keyword {key} duplicate values")
        return out

    # -- blocks ------------------------------------------------------------
    def block(self, key: str) -> Optional[List[str]]:
        """Lines between ``begin key`` and ``end key`` (units line included)."""
        ls = le = None
        for i, line in enumerate(self.data):
            if key in line and line.startswith("begin"):
                if ls is not None:
                    raise McinError(f"Found begin {key} more than once in input file")
                ls = i
        if ls is None:
            return None
        for i, line in enumerate(self.data):
            if key in line and line.startswith("end"):
                if le is not None:
                    raise McinError(f"Found end {key} more than once in input file")
                le = i
        if le is None:
            raise McinError(f"Found begin {key} but no end {key} in input file")
        if le <= ls:
            raise McinError(f"end {key} comes before begin {key} in input file")
        if len(_strip_all(self.data[ls])) != len(key) + 5:
            raise McinError(f"Unrecognised Begin block in {self.data[ls]} line")
        if len(_strip_all(self.data[le])) != len(key) + 3:
            raise McinError(f"Unrecognised End block in {self.data[le]} line")
        rows = self.data[ls + 1: le]
        for i in range(ls, le + 1):
            self.data[i] = ""
        return rows

    def leftovers(self) -> List[str]:
        return [d for d in self.data if d.strip()]


def _units_line(rows: List[str], nrows_expected: int, allow_energy: bool):
    """Optional units line of a block: returns (rows, bohr_length, ryd_energy)."""
    if len(rows) != nrows_expected + 1:
        return rows, False, False
    head = rows[0].strip()
    blen = ryd = False
    found_len = found_en = False
    for tok in [t for t in re.split(r"[\s,;:-]+", head) if t]:
        if tok in ("ang", "bohr"):
            if found_len:
                raise McinError("Found the length unit in block more than once")
            found_len, blen = True, tok == "bohr"
        elif tok in ("ev", "ryd") and allow_energy:
            if found_en:
                raise McinError("Found the energy unit in block more than once")
            found_en, ryd = True, tok == "ryd"
        else:
            raise McinError(f"Units in block not recognised: {head}")
    return rows[1:], blen, ryd


def _recip_lattice(real_lat: np.ndarray):
    """``utility_recip_lattice`` (utility.F90:44-83)."""
    r = real_lat
    rec = np.empty((3, 3))
    rec[0, 0] = r[1, 1] * r[2, 2] - r[2, 1] * r[1, 2]
    rec[0, 1] = r[1, 2] * r[2, 0] - r[2, 2] * r[1, 0]
    rec[0, 2] = r[1, 0] * r[2, 1] - r[2, 0] * r[1, 1]
    rec[1, 0] = r[2, 1] * r[0, 2] - r[0, 1] * r[2, 2]
    rec[1, 1] = r[2, 2] * r[0, 0] - r[0, 2] * r[2, 0]
    rec[1, 2] = r[2, 0] * r[0, 1] - r[0, 0] * r[2, 1]
    rec[2, 0] = r[0, 1] * r[1, 2] - r[1, 1] * r[0, 2]
    rec[2, 1] = r[0, 2] * r[1, 0] - r[1, 2] * r[0, 0]
    rec[2, 2] = r[0, 0] * r[1, 1] - r[1, 0] * r[0, 1]
    vol = r[0, 0] * rec[0, 0] + r[0, 1] * rec[0, 1] + r[0, 2] * rec[0, 2]
    if abs(vol) < EPS5:
        raise McinError("Found almost zero Volume in utility_recip_lattice")
    return TWOPI * rec / vol, abs(vol)


def frac_to_cart(frac, real_lat):
    """``utility_frac_to_cart``: cart(i) = sum_j real_lat(j,i) frac(j)."""
    return np.asarray(frac, dtype=float) @ real_lat


def cart_to_frac(cart, recip_lat):
    """``utility_cart_to_frac``: frac = recip_lat . cart / 2 pi."""
    return (recip_lat @ np.asarray(cart, dtype=float)) / TWOPI


def _snap_home(f: np.ndarray) -> np.ndarray:
    f = f.copy()
    for c in range(3):
        r = float(np.rint(f[c]))
        if abs(f[c] - r) < EPS5:
            f[c] = r
    return f - np.floor(f)


def _parse_pairs(L: _Lines, key: str, word: str, recip: np.ndarray,
                 want_shell: bool, want_sigma: bool) -> Optional[PairBlock]:
    """``param_get_parameters`` (parameters.F90:2558-2846)."""
    rows = L.block(key)
    if rows is None:
        return None
    # a units line is recognised by the absence of a site definition
    bohr = ryd = False
    if rows and ("f1=" not in _strip_all(rows[0]) and "c1=" not in _strip_all(rows[0])):
        rows, bohr, ryd = _units_line(rows, len(rows) - 1, allow_energy=True)
    f1s, f2s, vals, shells, sigmas = [], [], [], [], []
    for raw in rows:
        d = _strip_all(raw)
        parts = d.split(":")
        if len(parts) < 3:
            raise McinError(f"param_read_parameters: malformed positions definition: {d}")
        sites = []
        for tag_i, p in zip(("1", "2"), parts[:2]):
            if p.startswith("c" + tag_i + "=") or ("c" + tag_i + "=") in p:
                xyz = np.array([_fnum(t) for t in _tokens(p.split("=", 1)[1])[:3]])
                if bohr:
                    xyz = xyz * BOHR
                sites.append(cart_to_frac(xyz, recip))
            elif ("f" + tag_i + "=") in p:
                sites.append(np.array([_fnum(t) for t in _tokens(p.split("=", 1)[1])[:3]]))
            else:
                raise McinError(f"param_get_parameters: Atom site not recognised {p}")
        if (word + "=") not in parts[2]:
            raise McinError(f"param_read_parameters: malformed parameters definition: {d}")
        v = _fnum(parts[2].split("=", 1)[1])
        sh = sg = None
        nsh = nsg = 0
        for extra in parts[3:]:
            if extra.startswith("sh="):
                sh = _fnum(extra[3:]); nsh += 1
            elif extra.startswith("sig="):
                sg = _fnum(extra[4:]); nsg += 1
        if want_shell and nsh != 1:
            raise McinError(f"param_get_parameters: lspincorr is true but no shell is found in {key} block")
        if want_sigma and nsg != 1:
            raise McinError(f"param_get_parameters: spin_glass is true but no sigma is found in {key} block")
        f1s.append(sites[0]); f2s.append(sites[1]); vals.append(v)
        shells.append(sh if sh is not None else 0)
        sigmas.append(sg if sg is not None else 0.0)
    value = np.array(vals, dtype=float)
    sigma = np.array(sigmas, dtype=float)
    if ryd:
        value = value * HART * 0.5
        sigma = sigma * HART * 0.5
    return PairBlock(f1=np.array(f1s, dtype=float).reshape(-1, 3),
                     f2=np.array(f2s, dtype=float).reshape(-1, 3),
                     value=value,
                     shell=np.array(shells, dtype=int) if want_shell else None,
                     sigma=sigma if want_sigma else None)


def _parse_axes(L: _Lines, key: str, inp: McInput, with_param: bool):
    """``param_get_axes`` (parameters.F90:3061-3280) with lsort and lnorm."""
    rows = L.block(key)
    if rows is None:
        return None
    frac = "frac" in key
    rows, bohr, ryd = _units_line(rows, inp.num_atoms, allow_energy=with_param)
    if len(rows) != inp.num_atoms:
        raise McinError(f"Wrong number of lines in {key} block")
    labels, vecs, params = [], [], []
    for r in rows:
        t = _tokens(r)
        need = 5 if with_param else 4
        if len(t) < need:
            raise McinError(f"Problem reading block keyword {key}")
        labels.append(t[0])
        vecs.append([_fnum(x) for x in t[1:4]])
        params.append(_fnum(t[4]) if with_param else 0.0)
    vecs = np.array(vecs, dtype=float)
    params = np.array(params, dtype=float)
    if bohr:
        vecs = vecs * BOHR
    if ryd:
        params = params * HART * 0.5
    if frac:
        vecs = np.array([frac_to_cart(v, inp.real_lattice) for v in vecs])
    # sort according to the species order of the atoms block
    out_v, out_p = [], []
    for sym in inp.atoms_symbol:
        for a in range(inp.num_atoms):
            if labels[a] == sym:
                out_v.append(vecs[a]); out_p.append(params[a])
    if len(out_v) != inp.num_atoms:
        raise McinError(f"Wrong atoms symbol at the block keyword {key}")
    out_v = np.array(out_v)
    for a in range(inp.num_atoms):
        if np.all(np.abs(out_v[a]) < EPS4):
            raise McinError(f"All component of an axe in block {key} are zero")
        out_v[a] = out_v[a] / math.sqrt(float(np.dot(out_v[a], out_v[a])))
    return out_v, np.array(out_p)


def parse_mcin(text: str, seedname: str = "", num_nodes: int = 1) -> McInput:
    """Parse the text of a ``seedname.mcin`` file (``param_read``)."""
    L = _Lines(text)
    inp = McInput(seedname=seedname)

    pu = L.keyword("parameter_unit") or "ev"
    if pu not in ("ev", "electronvolt") and not pu.startswith("ryd"):
        raise McinError("Value of parameter_unit not recognised in param_read")
    coordinate = L.keyword("coordinate") or "frac"
    if not (coordinate.startswith("frac") or coordinate.startswith("cart")):
        raise McinError("Value of coordinate not recognised in param_read")
    length_unit = L.keyword("length_unit") or "ang"
    if not (length_unit.startswith("ang") or length_unit == "bohr"):
        raise McinError("Value of length_unit not recognised in param_read")
    boundary = L.keyword("boundary") or "periodic"
    if not (boundary.startswith("peri") or boundary.startswith("open")):
        raise McinError("boundary not recognised in param_read")
    inp.boundary_open = boundary.startswith("open")
    for k in ("inputfile_setup1", "inputfile_setup2", "hamfile_setup"):
        if L.logical(k, False):
            raise McinError(f"{k}: the setup steps (-inp1/-inp2/-ham) are not part of the Monte Carlo path")

    inp.tems_mode = L.keyword("tems_mode") or "lin"
    if not any(inp.tems_mode.startswith(m) for m in ("man", "lin", "inv", "log")):
        raise McinError("tems_mode not recognised")
    inp.tem_start = L.real("tem_start", 5.0)
    inp.tem_end = L.real("tem_end", 5.0)
    inp.tems_num = L.integer("tems_num", 1)
    if inp.tems_num < 1:
        raise McinError("tems_num must be greater than zero")
    tv = L.vector("tems", inp.tems_num, _fnum)
    tems = np.zeros(inp.tems_num)
    if tv is not None:
        tems[:] = tv
    if not inp.tems_mode.startswith("man"):
        if inp.tem_start <= 0.0:
            raise McinError("tem_start must be greater than zero")
        if inp.tem_end <= 0.0:
            raise McinError("tem_end must be greater than zero")
        tems[0] = inp.tem_start
        n = inp.tems_num
        if n > 1:
            if inp.tems_mode.startswith("lin"):
                step = (inp.tem_end - inp.tem_start) / float(n - 1)
                tems = np.array([inp.tem_start + i * step for i in range(n)])
            elif inp.tems_mode.startswith("inv"):
                st = (1.0 / inp.tem_end - 1.0 / inp.tem_start) / float(n - 1)
                tems = np.array([1.0 / (1.0 / inp.tem_start + i * st) for i in range(n)])
            else:
                tems = np.array([inp.tem_start * math.exp(math.log(inp.tem_end / inp.tem_start)
                                                          * (1.0 * i / (n - 1))) for i in range(n)])
    else:
        if tv is None:
            raise McinError("tems_mode set to manual but no tems found")
        if np.any(tems <= 0.0):
            raise McinError("tems must be greater than zero")
    inp.tems = tems

    inp.steps_warmup = max(L.integer("steps_warmup", 100000), 0)
    inp.steps_mc = L.integer("steps_mc", 200000)
    if inp.steps_mc < 1:
        raise McinError("steps_mc must be greater than zero")
    inp.steps_measure = L.integer("steps_measure", 2)
    if inp.steps_measure < 0:
        raise McinError("steps_measure must be greater than zero")
    sc = L.vector("supercell_size", 3, _fint)
    inp.supercell_size = tuple(sc) if sc is not None else (4, 4, 4)
    if any(x < 1 for x in inp.supercell_size):
        raise McinError("supercell_size must be greater than zero")
    inp.initial_sconfig = L.keyword("initial_sconfig") or "ferro"
    if not any(inp.initial_sconfig.startswith(m) for m in ("ferro", "rand", "file")):
        raise McinError("Initial_sconfig not recognised")
    inp.mcarlo_mode = L.keyword("mcarlo_mode") or "random"
    if not (inp.mcarlo_mode.startswith("const") or inp.mcarlo_mode.startswith("rand")):
        raise McinError("mcarlo_mode not recognised")
    inp.tilt_angles_max = L.real("tilt_angles_max", 0.125)
    if inp.mcarlo_mode.startswith("const") and inp.tilt_angles_max < 0:
        raise McinError("tilt_angles_max must be positive")
    seeds = L.range_vector("seeds")
    if seeds is not None and len(seeds) != num_nodes:
        raise McinError("number of seeds should be equal to number of nodes")
    inp.seeds = seeds

    # unit cell
    rows = L.block("unit_cell_cart")
    if rows is None:
        raise McinError("Did not find the cell information in the input file")
    rows, bohr, _ = _units_line(rows, 3, allow_energy=False)
    if len(rows) != 3:
        raise McinError("Not correct the cell information in the input file")
    lat = np.array([[_fnum(t) for t in _tokens(r)[:3]] for r in rows], dtype=float)
    if bohr:
        lat = lat * BOHR
    inp.real_lattice = lat              # row k = lattice vector a_k
    inp.recip_lattice, inp.cell_volume = _recip_lattice(lat)

    # atoms
    rf, rc = L.block("atoms_frac"), L.block("atoms_cart")
    if rf is not None and rc is not None:
        raise McinError("Cannot specify both atoms_frac and atoms_cart")
    if rf is None and rc is None:
        raise McinError("No atoms_frac or atoms_cart block found")
    frac = rf is not None
    rows = rf if frac else rc
    labels, pos, mom = [], [], []
    bohr = False
    if rows and len(_tokens(rows[0])) == 1:
        head = rows[0].strip()
        if head not in ("ang", "bohr"):
            raise McinError("Units in block atoms not recognised")
        bohr = head == "bohr"
        rows = rows[1:]
    for r in rows:
        t = _tokens(r)
        if len(t) < 5:
            raise McinError("Problem reading block keyword atoms")
        labels.append(t[0]); pos.append([_fnum(x) for x in t[1:4]]); mom.append(_fnum(t[4]))
    if not labels:
        raise McinError("No atom positions specified")
    pos = np.array(pos, dtype=float)
    if not frac:
        if bohr:
            pos = pos * BOHR
        pos = np.array([cart_to_frac(p, inp.recip_lattice) for p in pos])
    pos = np.array([_snap_home(p) for p in pos])
    mom = np.array(mom, dtype=float)
    if np.any(mom == 0.0):
        raise McinError("mag_moments can not be zero")
    species: List[str] = []
    for lb in labels:
        if lb not in species:
            species.append(lb)
    order = [a for sp in species for a in range(len(labels)) if labels[a] == sp]
    inp.num_atoms = len(labels)
    inp.num_species = len(species)
    inp.atoms_label = species
    inp.atoms_symbol = [sp[:3] for sp in species]
    inp.atoms_species_num = [labels.count(sp) for sp in species]
    inp.atoms_frac = pos[order]
    inp.atoms_cart = np.array([frac_to_cart(p, inp.real_lattice) for p in inp.atoms_frac])
    inp.mag_cell = mom[order]
    inp.atom_species = [species.index(labels[a]) for a in order]
    convert = order  # species-major position -> original row

    L.real("neighbors_tol", 0.001)
    inp.lstaggered = L.logical("staggered_m", False)
    if inp.lstaggered and inp.num_atoms == 1:
        inp.lstaggered = False
    # staggered_m_coeff (parameters.F90:450-463): +1 by default, only +1/-1,
    # reordered with the atoms (matmul with convert_matrix_atoms)
    coeff = L.vector("staggered_m_coeff", inp.num_atoms, _fint)
    if inp.lstaggered and coeff is not None and any(abs(int(c)) != 1 for c in coeff):
        raise McinError("Error: staggered_m_coeff must be +1 or -1")
    if coeff is None:
        coeff = [1] * inp.num_atoms
    inp.staggered_coeff = np.array([int(coeff[c]) for c in convert])
    inp.lorderparam = L.logical("order_parameter", False)
    for k in ("order_parameter_axes_frac", "order_parameter_axes_cart"):
        ax = _parse_axes(L, k, inp, with_param=False)
        if ax is not None:
            inp.orderparam_axes_cart = ax[0]
    if inp.lorderparam and inp.orderparam_axes_cart is None:
        raise McinError("No order_parameter_axes_frac or order_parameter_axes_cart block found")

    inp.lbinerror = L.logical("binning_error", False)
    bl = L.range_vector("binning_level")
    inp.binning_level = bl if bl is not None else [1, 2, 3, 4, 5]
    if inp.lbinerror and (any(b <= 0 for b in inp.binning_level)
                          or any(inp.steps_mc // (2 ** b) <= 1 for b in inp.binning_level)):
        raise McinError("binning_level contain non-valid numbers. It must be greater than zero "
                        "and as (steps_mc/2^(binning_level))-1>0.")
    inp.lspincorr = L.logical("spin_correlation", False)
    inp.energy_write = L.logical("energy_write", False)
    inp.energy_num_print = L.integer("energy_num_print", 1000)
    if inp.energy_num_print < 1:
        raise McinError("energy_num_print must be greater than zero")
    # structure factor (parameters.F90:543-592): fractional vectors converted
    # to cartesian with the reciprocal lattice (rows b_j, 2 pi included)
    inp.lsfactor = L.logical("sfactor", False)
    defaults = {"sfactor_polar": [1.0, 0.0, 0.0], "sfactor_corner": [0.0, 0.0, 0.0],
                "sfactor_q1": [1.0, 0.0, 0.0], "sfactor_q2": [0.0, 0.0, 1.0]}
    for k, d in defaults.items():
        v = L.vector(k, 3, _fnum)
        if k == "sfactor_polar":
            inp.lsfactor_polar = v is not None
        setattr(inp, k, np.asarray(v if v is not None else d, dtype=float) @ inp.recip_lattice)
    if np.linalg.norm(np.cross(inp.sfactor_q1, inp.sfactor_q2)) < 1e-8:
        raise McinError("Error: Vectors sfactor_q1 and sfactor_q2 not linearly independent")
    inp.sfactor_steps_measure = L.integer("sfactor_steps_measure", 100)
    if inp.lsfactor and (inp.sfactor_steps_measure < 1 or inp.sfactor_steps_measure > inp.steps_mc):
        raise McinError("Error: sfactor_steps_measure must be greater than zero and less than steps_mc.")
    mesh = L.vector("sfactor_2dqmesh", 2, _fint)
    inp.sfactor_2dqmesh = [int(x) for x in mesh] if mesh is not None else [50, 50]
    if inp.lsfactor and any(x < 1 for x in inp.sfactor_2dqmesh):
        raise McinError("Error: sfactor_2dqmesh must be greater than zero")

    inp.pt = L.logical("pt", False)
    if inp.pt and inp.tems_num <= 1:
        raise McinError("tems_num must be greater than one in parallel tempering algorithm")
    if inp.pt:
        inp.tems = np.sort(inp.tems)          # utility_sort, parameters.F90:601
    inp.pt_steps_swap = L.integer("pt_steps_swap", 1)
    if inp.pt and inp.pt_steps_swap < 1:
        raise McinError("pt_steps_swap must be greater than zero")
    if inp.pt and inp.energy_write and inp.pt_steps_swap > inp.energy_num_print:
        inp.energy_num_print = inp.pt_steps_swap
    inp.pt_print_swap = L.integer("pt_print_swap", 10000)
    if inp.pt and inp.pt_print_swap < 1:
        raise McinError("pt_print_swap must be greater than zero")
    inp.spin_glass = L.logical("spin_glass", False)
    L.integer("spin_glass_seed", 0)

    # setup-mode shell blocks: accepted and ignored at Monte Carlo time
    L.integer("shells_jij", 1)
    L.block("parameters_jij")
    inp.have_biquad = L.logical("ham_bij", False)
    L.integer("shells_bij", 0)
    L.block("parameters_bij")
    inp.have_dm = L.logical("ham_dij", False)
    L.integer("shells_dij", 0)
    L.block("parameters_dij")

    inp.jij = _parse_pairs(L, "jij_parameters", "jij", inp.recip_lattice,
                           want_shell=inp.lspincorr, want_sigma=inp.spin_glass)
    if inp.jij is None:
        raise McinError("param_read: no jij_parameters block found")
    inp.bij = _parse_pairs(L, "bij_parameters", "bij", inp.recip_lattice, False, False)
    if inp.have_biquad and inp.bij is None:
        raise McinError("param_read: ham_bij is true but no bij_parameters block found")
    inp.dij = _parse_pairs(L, "dij_parameters", "dij", inp.recip_lattice, False, False)
    if inp.have_dm and inp.dij is None:
        raise McinError("param_read: ham_dij is true but no dij_parameters block found")
    vf, vc = L.block("dij_vectors_frac"), L.block("dij_vectors_cart")
    if vf is not None and vc is not None:
        raise McinError("Cannot specify both dij_vectors_frac and dij_vectors_cart")
    if inp.have_dm and vf is None and vc is None:
        raise McinError("no dij_vectors_frac or dij_vectors_cart block found")
    if vf is not None or vc is not None:
        nd = 0 if inp.dij is None else len(inp.dij.value)
        rows = vf if vf is not None else vc
        rows, bohr, _ = _units_line(rows, nd, allow_energy=False)
        if len(rows) != nd:
            raise McinError("Wrong number of lines in dij_vectors_cart or dij_vectors_frac block")
        vecs = np.array([[_fnum(t) for t in _tokens(r)[:3]] for r in rows], dtype=float).reshape(-1, 3)
        if bohr:
            vecs = vecs * BOHR
        if vf is not None:
            vecs = np.array([frac_to_cart(v, inp.real_lattice) for v in vecs]).reshape(-1, 3)
        if inp.have_dm:
            for i in range(len(vecs)):
                if np.all(np.abs(vecs[i]) < EPS4):
                    raise McinError("dij_vectors cannot be zero")
                vecs[i] = vecs[i] / math.sqrt(float(np.dot(vecs[i], vecs[i])))
        inp.dij_vectors_cart = vecs

    inp.have_singleion = L.logical("ham_singleion", False)
    sf = _parse_axes(L, "singleion_axes_frac", inp, with_param=True)
    sca = _parse_axes(L, "singleion_axes_cart", inp, with_param=True)
    if sf is not None and sca is not None:
        raise McinError("Cannot specify both singleion_axes_frac and singleion_axes_cart")
    ax = sf if sf is not None else sca
    if inp.have_singleion and ax is None:
        raise McinError("ham_singeleion is true but no singleion_axes_frac or singleion_axes_cart block found")
    if ax is not None:
        inp.singleion_axes_cart = ax[0]
        inp.singleion_parameters = ax[1] / K_B

    inp.have_field = L.logical("ham_field", False)
    ff = _parse_axes(L, "field_axes_frac", inp, with_param=True)
    fc = _parse_axes(L, "field_axes_cart", inp, with_param=True)
    if ff is not None and fc is not None:
        raise McinError("Cannot specify both field_axes_frac and field_axes_cart")
    ax = ff if ff is not None else fc
    if inp.have_field and ax is None:
        raise McinError("singeleion is true but no field_axes_frac or field_axes_cart found")
    if ax is not None:
        inp.field_axes_cart = ax[0]
        inp.field_parameters = ax[1] * BOHR_MAGN / K_B

    left = L.leftovers()
    if left:
        raise McinError("Unrecognised keyword(s) in input file:\n" + "\n".join(left))
    return inp


def read_mcin(path: str, num_nodes: int = 1) -> McInput:
    import os
    seed = os.path.basename(path)
    if seed.endswith(".mcin"):
        seed = seed[: -len(".mcin")]
    with open(path, "r") as fh:
        return parse_mcin(fh.read(), seedname=seed, num_nodes=num_nodes)
