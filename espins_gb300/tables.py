"""Supercell pair expansion into ELL tables, as the reference builds them.

The reference expands each per-cell pair row (f1, f2, value) over every cell of
the supercell and stores the result as site-fastest ELL arrays
(ESpinS ``src/jij.F90:196-318`` expansion, ``:394-446`` compaction;
``src/bij.F90:145-359``; ``src/dij.F90:145-391``):

* site numbering ``i = cell*num_atoms + atom`` with cells x-fastest and atoms
  species-major (jij.F90:179-189, 219, 229);
* fractional coordinates within 1e-5 of an integer are snapped to it, cells
  wrap with ``mod(l + 10 L, L)`` and atoms match within 1e-4 (jij.F90:200-245);
* ``boundary = open`` drops a bond whose second atom falls in cell index -1 or
  L along any axis (jij.F90:264-267) -- the slot is still consumed;
* values are divided by ``|m_i m_j|`` (jij.F90:290-291, bij.F90:237-238,
  dij.F90:237-239); entries whose value is exactly zero are dropped when the
  per-site lists are compacted, and the remaining entries keep the order in
  which the (cell, pair) loops produced them.

Outputs use 0-based neighbour indices; :func:`to_fortran` turns them into the
1-based arrays a Fortran host holds (``jij_nbors_matrix(N,maxnb)`` etc.).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Optional

import numpy as np

from .mcin import EPS4, EPS5, K_B, McInput, McinError


@dataclass
class EllTable:
    """One interaction table in ELL form (0-based, site-fastest)."""
    nn: np.ndarray      # (N,) int32 neighbour counts
    nb: np.ndarray      # (maxnb, N) int32 neighbour site indices
    val: np.ndarray     # (maxnb, N) float64, or (maxnb, N, 3) for DM

    @property
    def maxnb(self) -> int:
        return int(self.nb.shape[0])


@dataclass
class Hamiltonian:
    """Everything the Monte Carlo kernels read (all energies in Kelvin)."""
    n: int
    num_atoms: int
    supercell: tuple
    mag: np.ndarray                     # (N,) signed moments
    jij: EllTable
    bij: Optional[EllTable] = None
    dij: Optional[EllTable] = None
    si_axis: Optional[np.ndarray] = None   # (num_atoms, 3)
    si_delta: Optional[np.ndarray] = None  # (num_atoms,)
    field_axis: Optional[np.ndarray] = None
    field_val: Optional[np.ndarray] = None


def _snap(x: np.ndarray) -> np.ndarray:
    r = np.rint(x)
    return np.where(np.abs(x - r) < EPS5, r, x)


def _find_atom(pos: np.ndarray, atoms_frac: np.ndarray) -> np.ndarray:
    """Index of the first atom within 1e-4 in every component, -1 if none."""
    out = np.full(pos.shape[0], -1, dtype=np.int64)
    for a in range(atoms_frac.shape[0] - 1, -1, -1):
        hit = np.all(np.abs(pos - atoms_frac[a][None, :]) <= EPS4, axis=1)
        out = np.where(hit, a, out)
    return out


def _expand_sites(num_atoms: int, atoms_frac: np.ndarray, supercell, open_boundary: bool,
                  f1: np.ndarray, f2: np.ndarray, what: str):
    """First and second site of every (cell, pair row), in the visiting order
    of the reference loops (cell outer, pair inner), with the open-boundary
    keep mask and the pair row of each entry."""
    L = np.asarray(supercell, dtype=np.int64)
    ncell = int(L[0] * L[1] * L[2])
    n = ncell * num_atoms
    npairs = f1.shape[0]
    cells = np.arange(ncell, dtype=np.int64)
    lmn = np.stack([cells % L[0], (cells // L[0]) % L[1], cells // (L[0] * L[1])], axis=1).astype(float)

    i1_all = np.empty((ncell, npairs), dtype=np.int64)
    i2_all = np.empty((ncell, npairs), dtype=np.int64)
    keep_all = np.empty((ncell, npairs), dtype=bool)
    for p in range(npairs):
        a1 = _snap(f1[p][None, :] + lmn)
        l1 = np.floor(a1).astype(np.int64)
        at1 = _find_atom(a1 - l1, atoms_frac)
        if np.any(at1 < 0):
            raise McinError(f"Unrecognised Atomic Position found in {what}_parameters block")
        w = (l1 + 10 * L[None, :]) % L[None, :]
        c1 = w[:, 2] * L[1] * L[0] + w[:, 1] * L[0] + w[:, 0]
        a2 = _snap(f2[p][None, :] + lmn)
        l2 = np.floor(a2).astype(np.int64)
        keep = np.ones(ncell, dtype=bool)
        if open_boundary:
            keep = ~np.any((l2 < 0) | (l2 == L[None, :]), axis=1)
        at2 = _find_atom(a2 - l2, atoms_frac)
        if np.any(at2[keep] < 0):
            raise McinError(f"Unrecognised Atomic Position found in {what}_parameters block")
        w2 = (l2 + 10 * L[None, :]) % L[None, :]
        c2 = w2[:, 2] * L[1] * L[0] + w2[:, 1] * L[0] + w2[:, 0]
        i1_all[:, p] = c1 * num_atoms + at1
        i2_all[:, p] = np.where(keep, c2 * num_atoms + np.maximum(at2, 0), 0)
        keep_all[:, p] = keep
    # visiting order of the reference loops: cell outer, pair inner
    return i1_all.reshape(-1), i2_all.reshape(-1), keep_all.reshape(-1), np.tile(np.arange(npairs), ncell), n


def expand_pairs(num_atoms: int, atoms_frac: np.ndarray, mag_cell: np.ndarray,
                 supercell, open_boundary: bool, f1: np.ndarray, f2: np.ndarray,
                 values: np.ndarray, what: str = "Jij") -> EllTable:
    """Expand pair rows over the supercell and compact into ELL.

    ``values`` has shape (npairs,) for J/B or (npairs, 3) for D (already in K).
    """
    vec = values.ndim == 2
    i1f, i2f, kf, pidx, n = _expand_sites(num_atoms, atoms_frac, supercell, open_boundary, f1, f2, what)
    mm = np.abs(mag_cell[i1f % num_atoms] * mag_cell[i2f % num_atoms])
    if vec:
        v = values[pidx] / mm[:, None]
        nz = np.any(v != 0.0, axis=1) & kf
    else:
        v = values[pidx] / mm
        nz = (v != 0.0) & kf
    order = np.argsort(i1f, kind="stable")
    i1s, i2s, nzs, vs = i1f[order], i2f[order], nz[order], v[order]
    sel = nzs
    i1s, i2s, vs = i1s[sel], i2s[sel], vs[sel]
    nn = np.bincount(i1s, minlength=n).astype(np.int32)
    maxnb = int(nn.max()) if n > 0 and nn.size else 0
    starts = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(nn, out=starts[1:])
    k = np.arange(i1s.size, dtype=np.int64) - starts[i1s]
    nb = np.zeros((maxnb, n), dtype=np.int32)
    nb[k, i1s] = i2s
    if vec:
        val = np.zeros((maxnb, n, 3), dtype=np.float64)
        val[k, i1s, :] = vs
    else:
        val = np.zeros((maxnb, n), dtype=np.float64)
        val[k, i1s] = vs
    return EllTable(nn=nn, nb=nb, val=val)


@dataclass
class ShellTables:
    """Neighbour shells of spincorr_get (jij.F90:449-503), 0-based.

    kind[i]            species of site i (kind_atoms)
    nn[s, i]           neighbours of site i in shell s+1 (shell_num_nbors_matrix)
    nb[s, k, i]        k-th such neighbour, in the order of the Jij rows
                       (shell_nbors_matrix)
    count[s, a, b]     shell_num_nbors_kind(s+1, a+1, b+1): the shell-(s+1)
                       neighbours of species a around the LAST site of
                       species b, as jij.F90:478-479 leaves it
    """
    kind: np.ndarray
    nn: np.ndarray
    nb: np.ndarray
    count: np.ndarray
    num_species: int

    @property
    def num_shells(self) -> int:
        return int(self.nn.shape[0])


def build_shells(inp: McInput) -> ShellTables:
    """shell_neighbors_get over the expanded Jij rows: every (cell, row) entry
    whose row carries shell sh > 0 and whose second site exists (open
    boundaries drop it) lists the second site under shell sh of the first."""
    j = inp.jij
    if j.shell is None:
        raise McinError("spin_correlation needs a shell (sh=) on every Jij_parameters row")
    S = int(np.max(j.shell))
    n = inp.num_total_atoms
    nsp = len(inp.atoms_symbol)
    kind = np.tile(np.asarray(inp.atom_species, dtype=np.int32), inp.num_supercell)
    i1f, i2f, kf, pidx, _ = _expand_sites(inp.num_atoms, inp.atoms_frac, inp.supercell_size,
                                          inp.boundary_open, j.f1, j.f2, "Jij")
    sh = np.asarray(j.shell, dtype=np.int64)[pidx]
    sel = kf & (sh > 0)
    order = np.argsort(i1f, kind="stable")          # per first site, in row order
    order = order[sel[order]]
    i1s, i2s, ss = i1f[order], i2f[order], sh[order] - 1
    nn = np.zeros((S, n), dtype=np.int32)
    np.add.at(nn, (ss, i1s), 1)
    maxk = int(nn.max()) if nn.size else 0
    nb = np.zeros((S, max(maxk, 1), n), dtype=np.int32)
    # position of every entry within its (shell, site) list
    key = ss * n + i1s
    o2 = np.argsort(key, kind="stable")
    ks = key[o2]
    first = np.searchsorted(ks, ks, side="left")
    pos = np.empty_like(o2)
    pos[o2] = np.arange(o2.size) - first
    nb[ss, pos, i1s] = i2s
    count = np.zeros((S, nsp, nsp), dtype=np.int32)
    for b in range(nsp):
        sites = np.nonzero(kind == b)[0]
        if sites.size == 0:
            continue
        last = sites[-1]
        for s_ in range(S):
            nbrs = nb[s_, :nn[s_, last], last]
            count[s_, :, b] = np.bincount(kind[nbrs], minlength=nsp)
    return ShellTables(kind=kind, nn=nn, nb=nb, count=count, num_species=nsp)


def site_positions(inp: McInput) -> np.ndarray:
    """Cartesian position of every site (mcarlo_get_atoms_pos,
    get_quant.F90:600-646): atom fractional position plus its cell's integer
    offset, cells x-fastest, atoms species-major."""
    L = np.asarray(inp.supercell_size, dtype=np.int64)
    ncell = int(L.prod())
    cells = np.arange(ncell)
    lmn = np.stack([cells % L[0], (cells // L[0]) % L[1], cells // (L[0] * L[1])], axis=1).astype(float)
    frac = (lmn[:, None, :] + np.asarray(inp.atoms_frac, dtype=float)[None, :, :]).reshape(-1, 3)
    return frac @ inp.real_lattice


def sfactor_qpoints(inp: McInput) -> np.ndarray:
    """The q-points of mcarlo_structure_factor (get_quant.F90:670-685), in
    loop_xy order: corner + (i/m1) q1 + (j/m2) q2 for i = 0..m1 (slow),
    j = 0..m2 (fast); cartesian, 1/length."""
    m1, m2 = inp.sfactor_2dqmesh
    out = np.empty(((m1 + 1) * (m2 + 1), 3))
    for xy in range(out.shape[0]):
        lx, ly = xy // (m2 + 1), xy % (m2 + 1)
        out[xy] = inp.sfactor_corner + (lx / float(m1)) * inp.sfactor_q1 + (ly / float(m2)) * inp.sfactor_q2
    return out


def check_symmetric(t: EllTable, antisym: bool, what: str) -> None:
    """The periodic-boundary symmetry checks of jij.F90:323-371 / dij.F90:285."""
    n = t.nn.shape[0]
    for i in range(n):
        for k in range(int(t.nn[i])):
            j = int(t.nb[k, i])
            ks = [kk for kk in range(int(t.nn[j])) if t.nb[kk, j] == i]
            if not ks:
                raise McinError(f"Found asymmetric pairs in {what}_parameters block ({i + 1},{j + 1})")
            a = t.val[k, i]
            b = t.val[ks[0], j]
            bad = np.any(np.abs(a + b) > EPS4) if antisym else np.any(np.abs(a - b) > EPS4)
            if bad:
                raise McinError(f"Found asymmetric pairs in {what}_parameters block ({i + 1},{j + 1})")


def build_hamiltonian(inp: McInput, check: bool = True) -> Hamiltonian:
    """``jij_get`` / ``bij_get`` / ``dij_get`` plus the per-cell single-ion and field data."""
    if inp.spin_glass:
        raise McinError("spin_glass: random exchange is outside the Monte Carlo path of this build")
    n = inp.num_total_atoms
    mag = np.tile(inp.mag_cell, inp.num_supercell)
    j = inp.jij
    jt = expand_pairs(inp.num_atoms, inp.atoms_frac, inp.mag_cell, inp.supercell_size,
                      inp.boundary_open, j.f1, j.f2, j.value / K_B, "Jij")
    if check and not inp.boundary_open:
        check_symmetric(jt, False, "Jij")
    bt = dt = None
    if inp.have_biquad and inp.bij is not None:
        b = inp.bij
        bt = expand_pairs(inp.num_atoms, inp.atoms_frac, inp.mag_cell, inp.supercell_size,
                          inp.boundary_open, b.f1, b.f2, b.value / K_B, "Bij")
        if check and not inp.boundary_open:
            check_symmetric(bt, False, "Bij")
    if inp.have_dm and inp.dij is not None:
        d = inp.dij
        dv = inp.dij_vectors_cart * (d.value / K_B)[:, None]
        dt = expand_pairs(inp.num_atoms, inp.atoms_frac, inp.mag_cell, inp.supercell_size,
                          inp.boundary_open, d.f1, d.f2, dv, "Dij")
        if check and not inp.boundary_open:
            check_symmetric(dt, True, "Dij")
    h = Hamiltonian(n=n, num_atoms=inp.num_atoms, supercell=tuple(inp.supercell_size),
                    mag=mag, jij=jt, bij=bt, dij=dt)
    if inp.have_singleion:
        h.si_axis = np.asarray(inp.singleion_axes_cart, dtype=float)
        h.si_delta = np.asarray(inp.singleion_parameters, dtype=float)
    if inp.have_field:
        h.field_axis = np.asarray(inp.field_axes_cart, dtype=float)
        h.field_val = np.asarray(inp.field_parameters, dtype=float)
    return h


def to_fortran(t: EllTable):
    """(nn, nbors 1-based (N,maxnb) column-major, values) as a Fortran host holds them."""
    nb1 = (t.nb.astype(np.int32) + 1)
    nb1[np.arange(t.maxnb)[:, None] >= t.nn[None, :]] = 0
    return t.nn.astype(np.int32), nb1, t.val
