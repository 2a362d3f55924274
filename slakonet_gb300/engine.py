"""Host side of the GB300 path: parameter packing, batch planning, launches.

``TableSet`` packs a model's per-element-pair tables (the reference's
``Skf`` / ``SkfFeed`` data, slakonet/skf.py:152-199, slakonet/skfeed.py:560-739)
into one device buffer with an index, so the kernels read every integral
from HBM without the per-call Python feed.  ``plan_batch`` turns a list of
structures into the flat descriptor arrays of the C ABI (CSR over atoms,
atom pairs, k-points and (structure, k) problems).  ``Engine.run`` issues
the kernels on one stream: bonds -> phases -> real-space blocks -> Bloch
sums -> eigensolve -> Fermi/gap -> DOS.
"""
from __future__ import annotations

import copy
import ctypes
import math
import threading
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from . import _lib
from ._lib import call, ptr

H2E = 27.211
CUTOFF_BOHR = 10.0          # hs_matrix default (slakonet/slaterkoster.py:111)
KT_FERMI = 0.01             # fermi_search default (slakonet/fermi.py:143)

# stats record layout (mirrors csrc/fermi_dos.cu)
STAT = dict(mu_ha=0, fermi_ev=1, gap_ev=2, vbm_ev=3, cbm_ev=4, direct=5, vbm_k=6, cbm_k=7, vwidth=8,
            cwidth=9, min_dgap=10, direct_semi=11, efermi_ev=12, bandgap_ev=13, converged=14, iters=15,
            dos_fermi=16, dos_gapc=17, dos_total=18, metal=19, fallback=20, vbm_flat=21, cbm_flat=22,
            band_energy_ha=23)


def _dev(device) -> torch.device:
    d = torch.device(device)
    if d.type != "cuda":
        raise _lib.SknError("slakonet_gb300 runs on CUDA devices only (no CPU path)")
    return d


def _i32(a, device):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.int32)).to(device, non_blocking=True)


def _i64(a, device):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.int64)).to(device, non_blocking=True)


def _f64(a, device):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64)).to(device, non_blocking=True)


# ------------------------------------------------------------------ tables

class TableSet:
    """Device-resident packed SK tables for a set of species.

    ``h_tables[(za, zb)][(l1, l2)]`` / ``s_tables`` are tensors ``[l1+1, n_grid]``
    (live parameters are accepted; they are read, not copied, when
    ``requires_grad`` is off).  ``grids[(za, zb)]`` is the grid step,
    ``onsite[z]`` the per-l on-site energies, ``occupations[z]`` per shell.
    """

    def __init__(self, species: Sequence[int], shell_dict: Dict[int, List[int]], h_tables, s_tables, steps,
                 onsite, occupations, device):
        self.device = torch.device(device)
        self.species = [int(z) for z in sorted(set(int(z) for z in species))]
        self.sp_of = {z: i for i, z in enumerate(self.species)}
        nsp = len(self.species)
        self.shell_dict = {z: list(shell_dict[z]) for z in self.species}
        sp_nshell = np.zeros(nsp, np.int32)
        sp_shell_l = np.zeros(4 * nsp, np.int32)
        sp_norb = np.zeros(nsp, np.int32)
        for i, z in enumerate(self.species):
            ls = self.shell_dict[z]
            if len(ls) > 4 or any(l < 0 or l > 3 for l in ls):
                raise ValueError(f"at most 4 shells with l <= 3 per element, got {ls} for Z={z}")
            sp_nshell[i] = len(ls)
            sp_shell_l[4 * i: 4 * i + len(ls)] = ls
            sp_norb[i] = sum(2 * l + 1 for l in ls)
        tab_index = -np.ones(16 * nsp * nsp, np.int32)
        offs, ngrid, stepv, hs, ss = [], [], [], [], []
        self.param_slices = []   # (tensor, "H"|"S", offset, numel) in packing order
        off = 0
        for a, za in enumerate(self.species):
            for b, zb in enumerate(self.species):
                if (za, zb) not in h_tables:
                    continue
                for (l1, l2), th in sorted(h_tables[(za, zb)].items()):
                    ts = s_tables[(za, zb)][(l1, l2)]
                    if l1 > l2 or l2 > 3:
                        continue
                    t = len(offs)
                    tab_index[((a * nsp + b) * 4 + l1) * 4 + l2] = t
                    if th.shape[-1] < 9:
                        raise ValueError(f"table ({za},{zb},{l1},{l2}) has {th.shape[-1]} grid points; 9 needed")
                    if isinstance(th, torch.Tensor):
                        self.param_slices.append((th, "H", off, th.numel()))
                    if isinstance(ts, torch.Tensor):
                        self.param_slices.append((ts, "S", off, ts.numel()))
                    th = torch.as_tensor(th).detach().to(self.device, torch.float64)
                    ts = torch.as_tensor(ts).detach().to(self.device, torch.float64)
                    offs.append(off)
                    ngrid.append(th.shape[-1])
                    stepv.append(float(steps[(za, zb)]))
                    hs.append(th.reshape(-1))
                    ss.append(ts.reshape(-1))
                    off += th.numel()
        self.ntab = len(offs)
        self.tab_H = torch.cat(hs) if hs else torch.zeros(1, dtype=torch.float64, device=self.device)
        self.tab_S = torch.cat(ss) if ss else torch.zeros(1, dtype=torch.float64, device=self.device)
        self.tab_index = _i32(tab_index, self.device)
        self.tab_off = _i64(offs or [0], self.device)
        self.tab_ngrid = _i32(ngrid or [0], self.device)
        self.tab_step = _f64(stepv or [1.0], self.device)
        self.sp_nshell = _i32(sp_nshell, self.device)
        self.sp_shell_l = _i32(sp_shell_l, self.device)
        self.sp_norb_np = sp_norb
        self.sp_norb = _i32(sp_norb, self.device)
        # per-species orbital on-site energies and electron counts
        self.sp_onsite = []
        self.sp_nelec = np.zeros(nsp)
        for i, z in enumerate(self.species):
            e = np.asarray(onsite[z], dtype=np.float64)
            orb = []
            for l in self.shell_dict[z]:
                orb.extend([e[l]] * (2 * l + 1))
            self.sp_onsite.append(np.array(orb))
            self.sp_nelec[i] = float(np.sum(occupations[z]))

    def with_values(self) -> Optional["TableSet"]:
        """A TableSet with this one's layout and the current values of the tensors it was packed
        from (one concatenation each for H and S), or None when some table was not a tensor.
        This object is left unchanged, so engines still using it are unaffected."""
        lists = self.__dict__.get("_value_lists")
        if lists is None:
            hs = [t for t, kind, _, _ in self.param_slices if kind == "H"]
            ss = [t for t, kind, _, _ in self.param_slices if kind == "S"]
            lists = (hs, ss)
            self.__dict__["_value_lists"] = lists
        hs, ss = lists
        if len(hs) != self.ntab or len(ss) != self.ntab or self.ntab == 0:
            return None
        dev = self.device
        if any(t.device != dev or t.dtype != torch.float64 for t in (hs[0], ss[0], hs[-1], ss[-1])):
            flat = lambda t: t.detach().reshape(-1).to(dev, torch.float64)   # noqa: E731
        else:
            flat = lambda t: t.detach().view(-1)                             # noqa: E731
        new = copy.copy(self)
        with torch.no_grad():
            new.tab_H = torch.cat([flat(t) for t in hs])
            new.tab_S = torch.cat([flat(t) for t in ss])
        return new

    @classmethod
    def from_synthetic(cls, tables: dict, shell_dict, device):
        """From ``slakonet_gb300.synthetic.make_tables`` output."""
        steps = {k: tables["step"] for k in tables["pairs"]}
        h = {k: {kk: torch.as_tensor(vv) for kk, vv in v["H"].items()} for k, v in tables["pairs"].items()}
        s = {k: {kk: torch.as_tensor(vv) for kk, vv in v["S"].items()} for k, v in tables["pairs"].items()}
        onsite = {z: e["on_sites"] for z, e in tables["elements"].items()}
        occ = {z: e["occupations"] for z, e in tables["elements"].items()}
        species = sorted(tables["elements"].keys())
        sd = {z: list(shell_dict[z]) for z in species}
        return cls(species, sd, h, s, steps, onsite, occ, device)


# ---------------------------------------------------------------- planning

# The bond search gives each ordered atom pair one GPU thread that loops over every lattice translation
# of the structure's box, so its work is translations x atoms^2.  Both are bounded here: a 1 A cubic
# cell needs ~2,200 translations; the 1000-atom 5x5x5 zincblende supercell needs 125 x 10^6.
MAX_IMAGES = 1 << 20
MAX_PAIR_IMAGES = 10 ** 11


def check_structure(st: dict, cutoff: float = CUTOFF_BOHR, s: int = 0):
    """One structure's arrays (numbers, positions, cell, kpoints, weights) and its translation box,
    or ValueError when they disagree in length, hold non-finite values, or need an unbounded bond
    search.  Every flat offset the kernels use comes from these lengths, so a bad structure must
    stop here, on the host.  ``weights`` defaults to uniform."""
    z = np.asarray(st["numbers"], dtype=np.int64).reshape(-1)
    p = np.asarray(st["positions"], dtype=np.float64).reshape(-1, 3)
    c = np.asarray(st["cell"], dtype=np.float64).reshape(3, 3)
    k = np.asarray(st["kpoints"], dtype=np.float64).reshape(-1, 3)
    w = np.asarray(st.get("weights", np.full(len(k), 1.0 / max(len(k), 1))), dtype=np.float64).reshape(-1)
    _check_arrays(s, z, p, c, k, w)
    r = image_range(c, p, cutoff)
    n_img = int(np.prod(2 * r.astype(np.int64) + 1))
    if n_img > MAX_IMAGES or n_img * len(z) ** 2 > MAX_PAIR_IMAGES:
        raise ValueError(f"structure {s}: the cell is too small or too flat for the {cutoff:g} Bohr cutoff "
                         f"({'x'.join(str(2 * int(x) + 1) for x in r)} translations for {len(z)} atoms; "
                         f"at most {MAX_IMAGES} translations and {MAX_PAIR_IMAGES:.0e} atom-pair translations)")
    return z, p, c, k, w, r


def _check_arrays(s: int, z, p, c, k, w) -> None:
    if len(z) == 0:
        raise ValueError(f"structure {s}: no atoms")
    if len(p) != len(z):
        raise ValueError(f"structure {s}: {len(p)} positions for {len(z)} atoms")
    if len(k) == 0:
        raise ValueError(f"structure {s}: no k-points")
    if len(w) != len(k):
        raise ValueError(f"structure {s}: {len(w)} k-point weights for {len(k)} k-points")
    for name, a in (("positions", p), ("cell", c), ("kpoints", k), ("weights", w)):
        if not np.isfinite(a).all():
            raise ValueError(f"structure {s}: non-finite {name}")
    if abs(np.linalg.det(c)) <= 1e-12 * max(np.abs(c).max(), 1.0) ** 3:
        raise ValueError(f"structure {s}: singular cell")


INT32_LIMIT = 2 ** 31 - 1


def _check_index_range(n_at, orb_cum, nk, orb_ptr64) -> None:
    """The descriptor arrays hold batch-wide atom, orbital and k-point offsets in int32, and the
    Fermi/DOS kernels index one structure's nk x n_orbitals eigenvalues with an int."""
    if int(n_at.sum()) > INT32_LIMIT or int(orb_cum[-1]) > INT32_LIMIT or int(nk.astype(np.int64).sum()) > INT32_LIMIT:
        raise ValueError("batch too large: its atoms, orbitals and k-points must each total below 2^31")
    rows = nk.astype(np.int64) * np.diff(orb_ptr64).astype(np.int64)
    if (rows > INT32_LIMIT).any():
        s = int(np.argmax(rows > INT32_LIMIT))
        raise ValueError(f"structure {s}: {int(nk[s])} k-points x {int(rows[s] // max(int(nk[s]), 1))} orbitals "
                         "exceeds 2^31 eigenvalues")


def _checked_arrays(structures: Sequence[dict], cutoff: float):
    """check_structure for a whole batch: the per-structure loop only converts arrays and compares lengths;
    finiteness, singular cells and the translation boxes are computed once over the stacked arrays.  When
    anything looks wrong, the structures are checked one by one instead, so the first bad one raises
    check_structure's own error."""
    S = len(structures)
    nums, pos, cells, kp, kw = [], [], [], [], []
    try:
        for st in structures:
            z = np.asarray(st["numbers"], dtype=np.int64).reshape(-1)
            p = np.asarray(st["positions"], dtype=np.float64).reshape(-1, 3)
            c = np.asarray(st["cell"], dtype=np.float64).reshape(3, 3)
            k = np.asarray(st["kpoints"], dtype=np.float64).reshape(-1, 3)
            w = np.asarray(st["weights"] if "weights" in st else np.full(len(k), 1.0 / max(len(k), 1)),
                           dtype=np.float64).reshape(-1)
            if len(z) == 0 or len(p) != len(z) or len(k) == 0 or len(w) != len(k):
                raise ValueError
            nums.append(z)
            pos.append(p)
            cells.append(c)
            kp.append(k)
            kw.append(w)
        n_at = np.array([len(z) for z in nums], np.int64)
        C = np.stack(cells)
        P = np.concatenate(pos)
        ok = np.isfinite(C).all() and np.isfinite(P).all() and all(np.isfinite(k).all() for k in kp) and \
            all(np.isfinite(w).all() for w in kw)
        if not ok:
            raise ValueError
        det = np.linalg.det(C)
        if (np.abs(det) <= 1e-12 * np.maximum(np.abs(C).reshape(S, -1).max(1), 1.0) ** 3).any():
            raise ValueError
        inv = np.linalg.inv(C)
        first = np.concatenate([[0], np.cumsum(n_at)[:-1]])
        frac = np.einsum("ai,aij->aj", P, np.repeat(inv, n_at, axis=0))
        spread = np.maximum.reduceat(frac, first, axis=0) - np.minimum.reduceat(frac, first, axis=0)
        blen = np.linalg.norm(inv, axis=1)
        rng = (np.floor(cutoff * blen + spread) + 1).astype(np.int32)
        n_img = np.prod(2 * rng.astype(np.int64) + 1, axis=1)
        if (n_img > MAX_IMAGES).any() or (n_img * n_at ** 2 > MAX_PAIR_IMAGES).any():
            raise ValueError
    except (ValueError, KeyError, TypeError, IndexError, np.linalg.LinAlgError):
        # one structure at a time: the first bad one raises its own error
        out = [check_structure(st, cutoff, s) for s, st in enumerate(structures)]
        nums, pos, cells, kp, kw, r = (list(x) for x in zip(*out))
        rng = np.array(r, np.int32).reshape(S, 3)
    return nums, pos, cells, kp, kw, rng


def image_range(cell: np.ndarray, positions: np.ndarray, cutoff: float) -> np.ndarray:
    """Half-widths r of the translation box holding every bond shorter than cutoff.

    |T_a| < cutoff |b_a| + spread_a, with b_a the reciprocal vectors (without
    2 pi) and spread_a the extent of the fractional coordinates.
    """
    inv = np.linalg.inv(cell)
    frac = positions @ inv
    spread = frac.max(0) - frac.min(0) if len(frac) else np.zeros(3)
    blen = np.linalg.norm(inv, axis=0)
    return (np.floor(cutoff * blen + spread) + 1).astype(np.int32)


@dataclass
class Plan:
    n_struct: int
    numbers: List[np.ndarray]
    atom_ptr: np.ndarray
    orb_ptr: np.ndarray
    positions: np.ndarray
    cells: np.ndarray
    image_range: np.ndarray
    atom_species: np.ndarray
    atom_norb: np.ndarray
    atom_orb_off: np.ndarray
    orb_atom: np.ndarray
    onsite_H: np.ndarray
    pair_base: np.ndarray
    n_pairs: int
    pair_ni_nj: np.ndarray
    k_ptr: np.ndarray
    kpoints: np.ndarray
    kweights: np.ndarray
    kw_off: np.ndarray
    nk: np.ndarray
    nb: np.ndarray
    phase_base: np.ndarray
    n_phase: int
    prob_struct: np.ndarray
    prob_k: np.ndarray
    prob_n: np.ndarray
    hs_off: np.ndarray
    hs_total: int
    eig_off_prob: np.ndarray
    eig_off_struct: np.ndarray
    eig_total: int
    order: np.ndarray
    nelec: np.ndarray
    max_n: int
    # problems whose H(k), S(k) are exactly real: every component of 2k is an integer, so the
    # Bloch phases exp(i 2 pi k.T) are exactly +-1
    prob_real: Optional[np.ndarray] = None


def plan_batch(structures: Sequence[dict], tables: TableSet, cutoff: float = CUTOFF_BOHR) -> Plan:
    """Flat descriptors for a batch.  Each structure: numbers, positions (Bohr),
    cell (Bohr, rows = lattice vectors), kpoints [nk,3] fractional, optional weights.

    The per-structure loop only gathers arrays and sizes the translation box;
    everything per atom or per orbital is built with whole-batch array operations."""
    S = len(structures)
    if S == 0:
        raise ValueError("empty batch: no structures")
    nums, pos, cells, kp, kw, rng = _checked_arrays(structures, cutoff)
    n_at = np.array([len(z) for z in nums], np.int64)
    nk = np.array([len(k) for k in kp], np.int32)
    zall = np.concatenate(nums) if S else np.zeros(0, np.int64)
    lut = tables.__dict__.get("_species_lut")
    if lut is None:
        lut = np.full(max(tables.species) + 1, -1, np.int32)
        for z_, i in tables.sp_of.items():
            lut[z_] = i
        tables.__dict__["_species_lut"] = lut
    bad = (zall < 0) | (zall >= len(lut))
    species = np.where(bad, -1, lut[np.clip(zall, 0, len(lut) - 1)]).astype(np.int32)
    if (species < 0).any():
        raise ValueError(f"no parameters for element Z={int(zall[np.argmax(species < 0)])}")
    norb = tables.sp_norb_np[species].astype(np.int32)
    atom_ptr = np.zeros(S + 1, np.int32)
    atom_ptr[1:] = np.cumsum(n_at)
    atom_struct = np.repeat(np.arange(S), n_at)
    orb_cum = np.concatenate([[0], np.cumsum(norb, dtype=np.int64)])
    _check_index_range(n_at, orb_cum, nk, orb_cum[atom_ptr])
    orb_ptr = orb_cum[atom_ptr].astype(np.int32)
    nb = np.diff(orb_ptr).astype(np.int32)
    aoff = (orb_cum[:-1] - orb_ptr[atom_struct]).astype(np.int32)            # first local orbital per atom
    oatom = np.repeat(np.arange(len(zall)) - atom_ptr[atom_struct], norb).astype(np.int32)
    ons = tables.__dict__.get("_species_onsite_flat")
    if ons is None:
        ons = (np.concatenate([[0], np.cumsum([len(v) for v in tables.sp_onsite])]).astype(np.int64),
               np.concatenate(tables.sp_onsite) if tables.sp_onsite else np.zeros(0))
        tables.__dict__["_species_onsite_flat"] = ons
    first = np.repeat(ons[0][species], norb)                                   # per orbital: start of its species
    within = np.arange(int(orb_cum[-1])) - np.repeat(orb_cum[:-1], norb)       # orbital index within its atom
    onsite = ons[1][first + within] if len(first) else np.zeros(0)
    nelec = np.add.reduceat(tables.sp_nelec[species], atom_ptr[:-1]) if len(zall) else np.zeros(S)
    nelec = np.where(n_at > 0, nelec, 0.0).astype(np.float64)
    pair_sz = n_at * n_at
    pair_base = np.concatenate([[0], np.cumsum(pair_sz)[:-1]]).astype(np.int64)
    pb = int(pair_sz.sum())
    # norb_i * norb_j for every ordered atom pair, structure by structure
    ninj = np.concatenate([np.outer(norb[atom_ptr[s]:atom_ptr[s + 1]], norb[atom_ptr[s]:atom_ptr[s + 1]]).reshape(-1)
                           for s in range(S)]).astype(np.int64) if S else np.zeros(0, np.int64)
    k_ptr = np.zeros(S + 1, np.int32)
    k_ptr[1:] = np.cumsum(nk)
    nimg = np.prod(2 * rng.astype(np.int64) + 1, axis=1)
    ph_sz = nimg * nk
    phase_base = np.concatenate([[0], np.cumsum(ph_sz)[:-1]]).astype(np.int64)
    phb = int(ph_sz.sum())
    prob_struct = np.repeat(np.arange(S, dtype=np.int32), nk)
    prob_k = (np.arange(int(nk.sum()), dtype=np.int64) - np.repeat(k_ptr[:-1], nk)).astype(np.int32)
    prob_n = nb[prob_struct]
    sz = prob_n.astype(np.int64) ** 2
    hs_off = np.concatenate([[0], np.cumsum(sz)[:-1]]).astype(np.int64)
    eig_sz = nk.astype(np.int64) * nb
    eig_off_struct = np.concatenate([[0], np.cumsum(eig_sz)[:-1]]).astype(np.int64)
    eig_off_prob = eig_off_struct[prob_struct] + prob_k.astype(np.int64) * prob_n
    order = np.argsort(-prob_n, kind="stable").astype(np.int32)
    kw_off = k_ptr[:-1].astype(np.int64)
    kall = np.concatenate(kp) if S else np.zeros((0, 3))
    prob_real = np.all(2.0 * kall == np.round(2.0 * kall), axis=1)
    return Plan(S, nums, atom_ptr, orb_ptr, np.concatenate(pos) if S else np.zeros((0, 3)),
                np.stack(cells) if S else np.zeros((0, 3, 3)), rng, species, norb, aoff, oatom, onsite,
                pair_base, pb, ninj, k_ptr, kall, np.concatenate(kw) if S else np.zeros(0), kw_off,
                nk, nb, phase_base, phb, prob_struct, prob_k, prob_n, hs_off, int(sz.sum()),
                eig_off_prob, eig_off_struct, int(eig_sz.sum()), order, nelec, int(nb.max()) if S else 0,
                prob_real=prob_real)


# ------------------------------------------------------------------ engine

@dataclass
class BatchResult:
    plan: Plan
    eig: torch.Tensor            # flat eigenvalues, structure s at eig_off_struct[s], [nk][nb]
    eig_status: torch.Tensor     # per problem
    mu: torch.Tensor             # per structure (Hartree)
    stats: torch.Tensor          # [S, SKN_NSTAT]
    fermi_status: torch.Tensor
    dos_grid: torch.Tensor
    dos: torch.Tensor            # [S, npts]
    H: Optional[torch.Tensor] = None
    S: Optional[torch.Tensor] = None
    vec: Optional[torch.Tensor] = None   # complex128, problem p at hs_off[p], row-major [component][band]
    timings: dict = field(default_factory=dict)
    state: Optional[dict] = None

    def eigenvectors(self, s: int) -> torch.Tensor:
        """[nk, n, n] complex: [k, i, j] = component i of eigenvector j (ascending eigenvalues)."""
        p = self.plan
        n = int(p.nb[s])
        q = np.nonzero(p.prob_struct == s)[0]
        o = int(p.hs_off[q[0]])
        return self.vec[o: o + len(q) * n * n].view(len(q), n, n)

    def eigenvalues(self, s: int) -> torch.Tensor:
        p = self.plan
        o = int(p.eig_off_struct[s])
        return self.eig[o: o + int(p.nk[s]) * int(p.nb[s])].view(int(p.nk[s]), int(p.nb[s]))


BLOCH_KCHUNK = 8           # k-points per work unit of skn_bloch_pairs (csrc/bloch.cu)


class DeviceBatch:
    """A planned batch with its descriptor arrays resident on the device."""

    def __init__(self, plan: Plan, device):
        dev = device
        self.plan = plan
        self.atom_ptr = _i32(plan.atom_ptr, dev)
        self.pos = _f64(plan.positions, dev)
        self.cells = _f64(plan.cells, dev)
        self.rng = _i32(plan.image_range, dev)
        self.pair_base = _i64(plan.pair_base, dev)
        self.norb = _i32(plan.atom_norb, dev)
        self.kptr = _i32(plan.k_ptr, dev)
        self.kp = _f64(plan.kpoints, dev)
        self.phb = _i64(plan.phase_base, dev)
        self.species = _i32(plan.atom_species, dev)
        self.ps = _i32(plan.prob_struct, dev)
        self.pk = _i32(plan.prob_k, dev)
        self.hs_off = _i64(plan.hs_off, dev)
        self.orb_ptr = _i32(plan.orb_ptr, dev)
        self.orb_atom = _i32(plan.orb_atom, dev)
        self.aoff = _i32(plan.atom_orb_off, dev)
        self.onsite = _f64(plan.onsite_H, dev)
        self.n = _i32(plan.prob_n, dev)
        self.eoff = _i64(plan.eig_off_prob, dev)
        self.order = _i32(plan.order, dev)
        self.eos = _i64(plan.eig_off_struct, dev)
        self.nk = _i32(plan.nk, dev)
        self.nb = _i32(plan.nb, dev)
        self.kwoff = _i64(plan.kw_off, dev)
        self.kw = _f64(plan.kweights, dev)
        self.ne = _f64(plan.nelec, dev)
        # work units of the Bloch-sum kernel per structure: ceil(nk_s / BLOCH_KCHUNK) k-chunks times the
        # N_s^2 ordered atom pairs (full matrices) or the N_s (N_s + 1) / 2 pairs on or below the diagonal
        # (lower triangles), numbered from an exclusive prefix sum
        na = np.diff(plan.atom_ptr).astype(np.int64)
        kch = (plan.nk.astype(np.int64) + BLOCH_KCHUNK - 1) // BLOCH_KCHUNK

        def base(units):
            return _i64(np.concatenate([[0], np.cumsum(units)[:-1]]) if len(units) else np.zeros(1), dev), \
                int(units.sum())
        self.bloch_unit_base, self.bloch_units = base(na * na * kch)
        self.bloch_unit_base_lower, self.bloch_units_lower = base(na * (na + 1) // 2 * kch)

    def h2d_bytes(self) -> int:
        return sum(int(v.numel() * v.element_size()) for v in vars(self).values() if isinstance(v, torch.Tensor))


# kernels each ABI call launches (for the launch count the bench reports)
KERNELS_PER_CALL = {"skn_bond_counts": 1, "skn_bond_fill": 1, "skn_image_phases": 1, "skn_sk_blocks": 1,
                    "skn_bloch": 1, "skn_bloch_pairs": 1, "skn_eigh_gen_batched": 1, "skn_eigh_gen_vectors": 2, "skn_fermi_gap": 1,
                    "skn_dos": 2, "skn_eigh_gen_large": 1, "skn_eigh_gen_vectors_noalloc": 2}

def wide_launches(n: int, nb: int = 32, tc: bool = False, tc_min: int = 512) -> int:
    """Kernel launches of one skn_eigh_gen_wide(_tc) call for problems of n orbitals (its host sequence);
    with ``tc`` a rank-2k update of a trailing matrix of ``tc_min`` rows or more is two launches."""
    def r2k(m):
        return 2 if (tc and m >= tc_min) else 1
    T = -(-n // nb)
    k = 3 + T + (T - 1) + sum(r2k(n - c0 - nb) for c0 in range(0, n - nb, nb))    # set-up; Cholesky
    k += T + 3 * (T - 1) + sum(r2k(n - c0 - nb) for c0 in range(0, n - nb, nb))   # reduction
    k += (T - 1) + sum(1 for t in range(1, T) if (t + 1) * nb < n)   # deferred solves
    c0 = 0
    while c0 < n - 1:                         # tridiagonalisation: 6 per column, 1 per panel update
        w = min(nb, n - 1 - c0)
        k += 6 * w + (r2k(n - c0 - w) if n - c0 - w > 0 else 0)
        c0 += nb
    return k + 2                              # bounds and eigenvalues


_SIDE = threading.local()   # per-thread side streams of Engine._side_streams

SINGLE_CTA_MAX_N = 2048   # bound of the one-CTA-per-problem eigensolver (csrc/eigh.cu)
LARGE_MAX_N = 9216        # bound of the cluster eigensolver (csrc/eigh_cluster.cu)


def cluster_for(n: int) -> int:
    """CTAs (SMs) the cluster eigensolver gives one problem of n orbitals.

    Measured on GB300 (one problem alone, random Hermitian-definite pairs): at n = 1024
    one SM takes 3.5 s, clusters of 4/8/16 CTAs 0.78/0.61/0.53 s; at n = 2048 clusters of
    4/8/16 take 4.5/3.2/2.5 s; at n = 4096, 8/16 take 18.5/13.2 s.  Clusters that fit at
    once: 36 of 4 CTAs, 15 of 8, 8 of 12, 7 of 16.  Four CTAs keep most of the gain up to
    2048 orbitals; 8 up to 4096; above that 12, so that a structure's 8 k-points (a 2x2x2
    grid) all run at once."""
    return 4 if n <= 2048 else (8 if n <= 4096 else 12)


def route_wide(prob_n: np.ndarray, threshold: Optional[int]) -> np.ndarray:
    """True for problems the device-wide eigensolver takes (csrc/eigh_wide.cu): more than
    ``threshold`` orbitals (None: none).  Like route_large, the choice depends on each problem
    alone, and the wide path's results depend only on the problem, so a structure's results are
    bitwise the same whatever it is batched with."""
    if threshold is None:
        return np.zeros(len(prob_n), dtype=bool)
    return prob_n.astype(np.int64) > int(threshold)


def _default_tuning():
    """Launch shapes per size bucket when the engine has no autotuned ones (autotune.Tuning.default)."""
    from .autotune import Tuning
    return Tuning.default()


def launch_order(groups: Sequence[np.ndarray], prob_n: np.ndarray, prob_real: np.ndarray) -> List[int]:
    """Order in which the eigensolver's groups (arrays of problem indices) are launched.

    The groups run concurrently, each a persistent grid that takes every SM slot it can get, so a group
    whose CTAs reach the SMs second waits for the first group's CTAs to drain.  The group that must not
    wait is the one with a few long problems (on the benchmark batch, the ~100 real problems of up to 492
    orbitals): started last, they end ~130 ms after everything else.  So groups go by their largest
    problem's cost (n^3, x4 when complex) divided by the group's size: few long problems first, the many
    small ones last; ties keep the given order."""
    def urgency(i):
        sel = groups[i]
        cost = prob_n[sel].astype(np.float64) ** 3 * np.where(prob_real[sel], 1.0, 4.0)
        return -float(cost.max()) / len(sel)
    return sorted(range(len(groups)), key=urgency)


def route_large(prob_n: np.ndarray, threshold: Optional[int] = 1024, cluster: Optional[int] = None) -> np.ndarray:
    """Cluster size per problem, 0 for the one-CTA-per-problem eigensolver.

    Problems above ``threshold`` orbitals (and always those above SINGLE_CTA_MAX_N) go to
    the cluster eigensolver with ``cluster`` CTAs, or ``cluster_for(n)`` when it is None.
    The choice depends on each problem alone, never on the rest of the batch, so a
    structure's results are bitwise the same whatever it is batched with."""
    n = prob_n.astype(np.int64)
    mask = n > SINGLE_CTA_MAX_N
    if threshold is not None:
        mask |= n > int(threshold)
    sizes = np.zeros(len(n), dtype=np.int64)
    for i in np.nonzero(mask)[0]:
        sizes[i] = cluster if cluster is not None else cluster_for(int(n[i]))
    return sizes


class Engine:
    """Runs the whole path for a planned batch on one CUDA stream."""

    def __init__(self, tables: TableSet, cutoff: float = CUTOFF_BOHR, stream: Optional[torch.cuda.Stream] = None,
                 tuning=None, large_threshold: Optional[int] = 1024, large_cluster: Optional[int] = None,
                 real_path: bool = True, wide_threshold: Optional[int] = 1024, wide_tc: bool = True):
        _dev(tables.device)
        self.tables = tables
        self.tuning = tuning          # autotune.Tuning: eigensolver launch shape per problem-size bucket
        # which problems run on the cluster eigensolver and with how many CTAs (SMs) each:
        # see route_large (large_cluster None: cluster_for(n))
        self.large_threshold = large_threshold
        self.large_cluster = large_cluster
        # problems above wide_threshold orbitals run on the device-wide eigensolver instead (route_wide):
        # measured on GB300 it is 4.6x the 4-CTA cluster at n = 1024 and 6-7x at n = 2048-4096
        self.wide_threshold = wide_threshold
        # the device-wide path's rank-2k updates on the tensor cores (skn_eigh_gen_wide_tc): measured on
        # GB300, the 1000-atom structure (n = 9000, 8 real k-points) solves in 13.2 s instead of 18.9 s
        self.wide_tc = wide_tc
        # values-only solves of problems with exactly real H(k), S(k) use the real-arithmetic
        # kernel (skn_eigh_gen_batched_real): same numbers, a quarter of the FP64 work
        self.real_path = bool(real_path)
        self.cutoff = float(cutoff)
        self.device = tables.device
        self.stream = stream
        self.launches = 0
        self.event_log = None   # set to a list to record (name, start, end) CUDA events per call

    def _call(self, name, *args):
        ev = self.event_log
        if ev is not None:
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
        call(name, *args)
        if ev is not None:
            b.record()
            ev.append((name, a, b))
        self.launches += (wide_launches(args[1], tc=name.endswith("_tc")) if name.startswith("skn_eigh_gen_wide")
                          else KERNELS_PER_CALL.get(name, 1))

    def run(self, plan: Plan, dos_range=(-10.0, 10.0), dos_points: int = 5000, dos_sigma: float = 0.1,
            dos_window: float = 0.0, keep_hs: bool = False, hs_only: bool = False,
            vectors: bool = False) -> BatchResult:
        with torch.cuda.device(self.device):
            ctx = torch.cuda.stream(self.stream) if self.stream is not None else _nullctx()
            with ctx:
                db = DeviceBatch(plan, self.device)
                return self.execute(db, dos_range, dos_points, dos_sigma, dos_window, keep_hs, hs_only, vectors)

    def execute(self, db: DeviceBatch, dos_range=(-10.0, 10.0), dos_points: int = 5000, dos_sigma: float = 0.1,
                dos_window: float = 0.0, keep_hs: bool = False, hs_only: bool = False,
                vectors: bool = False, keep_state: bool = False) -> BatchResult:
        """Kernels only, on the current stream; one device->host read sizes the bond table."""
        bonds = self.bonds(db)
        return self.tail(db, bonds, dos_range, dos_points, dos_sigma, dos_window, keep_hs, hs_only, vectors,
                         keep_state)

    def bonds(self, db: DeviceBatch, out: Optional[dict] = None) -> dict:
        """Neighbour list: counts, host scan (one device->host read), fill.  The result is the
        structure-only part of the path and stays valid while the geometry does.  With ``out``
        (an earlier result for the same geometry, e.g. the buffers a captured graph reads) the
        list is rebuilt into those buffers; a count that differs from theirs raises."""
        plan = db.plan
        dev = self.device
        S = plan.n_struct
        stream = torch.cuda.current_stream(dev).cuda_stream
        counts = torch.empty(max(plan.n_pairs, 1), dtype=torch.int32, device=dev)
        self._call("skn_bond_counts", S, plan.n_pairs, ptr(db.atom_ptr), ptr(db.pos), ptr(db.cells), ptr(db.rng),
                   self.cutoff, ptr(db.pair_base), ptr(counts), stream)
        cnt = counts[: plan.n_pairs].to("cpu").numpy().astype(np.int64)
        pair_ptr = np.zeros(plan.n_pairs + 1, np.int64)
        np.cumsum(cnt, out=pair_ptr[1:])
        pair_blk = np.zeros(plan.n_pairs + 1, np.int64)
        np.cumsum(cnt * plan.pair_ni_nj, out=pair_blk[1:])
        nbond = int(pair_ptr[-1])
        nblk = int(pair_blk[-1])
        if out is not None:
            if out["nbond"] != nbond or out["nblk"] != nblk:
                raise ValueError("the neighbour list changed size: the geometry is not the captured one")
            b = out
            b["pair_ptr"].copy_(torch.from_numpy(pair_ptr), non_blocking=False)
            d_pair_blk = _i64(pair_blk[:-1] if plan.n_pairs else np.zeros(1), dev)
            d_pair_ptr = b["pair_ptr"]
        else:
            d_pair_ptr = _i64(pair_ptr, dev)
            d_pair_blk = _i64(pair_blk[:-1] if plan.n_pairs else np.zeros(1), dev)
            nb1 = max(nbond, 1)
            b = dict(nbond=nbond, nblk=nblk, pair_ptr=d_pair_ptr,
                     bond_i=torch.empty(nb1, dtype=torch.int32, device=dev),
                     bond_j=torch.empty(nb1, dtype=torch.int32, device=dev),
                     bond_img=torch.empty(nb1, dtype=torch.int32, device=dev),
                     bond_d=torch.empty(nb1, dtype=torch.float64, device=dev),
                     bond_u=torch.empty(3 * nb1, dtype=torch.float64, device=dev),
                     bond_blk=torch.empty(nb1, dtype=torch.int64, device=dev))
        self._call("skn_bond_fill", S, plan.n_pairs, ptr(db.atom_ptr), ptr(db.pos), ptr(db.cells), ptr(db.rng),
                   self.cutoff, ptr(db.pair_base), ptr(d_pair_ptr), ptr(d_pair_blk), ptr(db.norb), ptr(b["bond_i"]),
                   ptr(b["bond_j"]), ptr(b["bond_img"]), ptr(b["bond_d"]), ptr(b["bond_u"]), ptr(b["bond_blk"]),
                   stream)
        return b

    def tail(self, db: DeviceBatch, bonds: dict, dos_range=(-10.0, 10.0), dos_points: int = 5000,
             dos_sigma: float = 0.1, dos_window: float = 0.0, keep_hs: bool = False, hs_only: bool = False,
             vectors: bool = False, keep_state: bool = False) -> BatchResult:
        """Everything after the neighbour list; device work only (no host synchronisation), so
        it can be captured in a CUDA graph."""
        plan = db.plan
        dev = self.device
        T = self.tables
        S = plan.n_struct
        stream = torch.cuda.current_stream(dev).cuda_stream
        nbond, nblk = bonds["nbond"], bonds["nblk"]
        bond_i, bond_j, bond_img = bonds["bond_i"], bonds["bond_j"], bonds["bond_img"]
        bond_d, bond_u, bond_blk = bonds["bond_d"], bonds["bond_u"], bonds["bond_blk"]
        d_pair_ptr = bonds["pair_ptr"]
        phases = torch.empty(2 * max(plan.n_phase, 1), dtype=torch.float64, device=dev)
        self._call("skn_image_phases", S, ptr(db.rng), ptr(db.kptr), ptr(db.kp), ptr(db.phb), ptr(phases), stream)
        blk_H = torch.empty(max(nblk, 1), dtype=torch.float64, device=dev)
        blk_S = torch.empty(max(nblk, 1), dtype=torch.float64, device=dev)
        status = torch.zeros(1, dtype=torch.int32, device=dev)
        if nbond:
            self._call("skn_sk_blocks", nbond, ptr(bond_i), ptr(bond_j), ptr(bond_d), ptr(bond_u), ptr(bond_blk),
                       ptr(db.species), len(T.species), ptr(T.sp_nshell), ptr(T.sp_shell_l), ptr(T.sp_norb),
                       ptr(T.tab_index), ptr(T.tab_off), ptr(T.tab_ngrid), ptr(T.tab_step), ptr(T.tab_H),
                       ptr(T.tab_S), ptr(blk_H), ptr(blk_S), ptr(status), stream)
        n_prob = len(plan.prob_n)
        Hk = torch.empty(2 * max(plan.hs_total, 1), dtype=torch.float64, device=dev)
        Sk = torch.empty(2 * max(plan.hs_total, 1), dtype=torch.float64, device=dev)
        # the eigensolvers read only the lower triangles; full matrices only when they are returned
        lower = 0 if (keep_hs or hs_only) else 1
        self._call("skn_bloch_pairs", S, db.bloch_units_lower if lower else db.bloch_units,
                   ptr(db.bloch_unit_base_lower if lower else db.bloch_unit_base), ptr(db.kptr), ptr(db.hs_off),
                   ptr(db.atom_ptr),
                   ptr(db.orb_ptr), ptr(db.aoff), ptr(db.norb), ptr(db.pair_base), ptr(d_pair_ptr), ptr(bond_img),
                   ptr(bond_blk), ptr(blk_H), ptr(blk_S), ptr(db.rng), ptr(db.phb), ptr(phases), ptr(db.onsite),
                   lower, ptr(Hk), ptr(Sk), stream)
        self._status = status
        hs_copy = (Hk.clone(), Sk.clone()) if keep_hs else (None, None)
        if hs_only:
            self.check_tables()
            return BatchResult(plan, None, None, None, None, None, None, None, hs_copy[0], hs_copy[1])
        eig = torch.empty(max(plan.eig_total, 1), dtype=torch.float64, device=dev)
        eig_status = torch.empty(max(n_prob, 1), dtype=torch.int32, device=dev)
        counter = torch.zeros(2, dtype=torch.int32, device=dev)
        vec = None
        if vectors:
            vec = torch.empty(2 * max(plan.hs_total, 1), dtype=torch.float64, device=dev)
            tri = torch.empty(4 * max(plan.eig_total, 1), dtype=torch.float64, device=dev)
            need = ctypes.c_int64(0)
            call("skn_eigh_vectors_scratch_bytes", n_prob, plan.max_n, ctypes.addressof(need))
            scratch = torch.empty(max(need.value // 8, 1), dtype=torch.float64, device=dev)
            self._call("skn_eigh_gen_vectors", n_prob, ptr(db.n), ptr(db.hs_off), ptr(db.eoff), ptr(db.order),
                       ptr(Hk), ptr(Sk), ptr(eig), ptr(vec), ptr(eig_status), ptr(tri), ptr(scratch),
                       int(need.value), ptr(counter), plan.max_n, stream)
            vec = torch.view_as_complex(vec.view(-1, 2))
        else:
            ev = self.event_log
            if ev is not None:
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record()
                self.event_log = None        # the phase is timed as a whole (groups run on forked streams)
            self._eig_values(db, Hk, Sk, eig, eig_status, counter, stream)
            if ev is not None:
                b.record()
                self.event_log = ev
                ev.append(("eigensolve", a, b))
        mu = torch.empty(S, dtype=torch.float64, device=dev)
        stats = torch.zeros(S * _lib.SKN_NSTAT, dtype=torch.float64, device=dev)
        fst = torch.empty(S, dtype=torch.int32, device=dev)
        self._call("skn_fermi_gap", S, ptr(db.eos), ptr(db.nk), ptr(db.nb), ptr(db.kwoff), ptr(db.kw), ptr(db.ne),
                   ptr(eig), KT_FERMI, 1e-6, 100, ptr(mu), ptr(stats), ptr(fst), stream)
        grid = torch.empty(dos_points, dtype=torch.float64, device=dev)
        dos = torch.empty(S * dos_points, dtype=torch.float64, device=dev)
        self._call("skn_dos", S, ptr(db.eos), ptr(db.nk), ptr(db.nb), ptr(db.kwoff), ptr(db.kw), ptr(eig), ptr(mu),
                   float(dos_range[0]), float(dos_range[1]), int(dos_points), float(dos_sigma), float(dos_window),
                   ptr(grid), ptr(dos), ptr(stats), stream)
        out = BatchResult(plan, eig, eig_status, mu, stats.view(S, _lib.SKN_NSTAT), fst, grid,
                          dos.view(S, dos_points), hs_copy[0], hs_copy[1], vec)
        if keep_state:
            out.state = dict(bond_i=bond_i, bond_j=bond_j, bond_img=bond_img, bond_d=bond_d, bond_u=bond_u,
                             bond_blk=bond_blk, nbond=nbond, nblk=nblk, phases=phases, db=db,
                             dos_args=(float(dos_range[0]), float(dos_range[1]), int(dos_points), float(dos_sigma),
                                       float(dos_window)))
        return out

    def _eig_values(self, db, Hk, Sk, eig, eig_status, counter, stream):
        plan = db.plan
        n_prob = len(plan.prob_n)
        groups = self._groups(db)
        if not groups:
            self._call("skn_eigh_gen_batched", n_prob, ptr(db.n), ptr(db.hs_off), ptr(db.eoff), ptr(db.order),
                       ptr(Hk), ptr(Sk), ptr(eig), ptr(eig_status), ptr(counter), plan.max_n, stream)
            return
        scratch = {}
        for gi, (shape, _, count, max_n) in enumerate(groups):
            need = ctypes.c_int64(0)
            if isinstance(shape, int):       # a cluster group
                call("skn_eigh_large_scratch_bytes", count, max_n, shape, ctypes.addressof(need))
            elif isinstance(shape, tuple):   # a device-wide group: ("wide", n, real)
                call("skn_eigh_wide_scratch_bytes", count, max_n, ctypes.addressof(need))
            else:
                continue
            scratch[gi] = torch.empty(max(need.value // 8, 1), dtype=torch.float64, device=self.device)
        counters = torch.zeros(2 * len(groups), dtype=torch.int32, device=self.device)

        def launch(gi, sfx, order_g, count, max_n, st):
            if isinstance(sfx, tuple):
                self._call("skn_eigh_gen_wide_tc" if self.wide_tc else "skn_eigh_gen_wide", count, max_n,
                           ptr(order_g), ptr(db.n), ptr(db.hs_off), ptr(db.eoff),
                           ptr(Hk), ptr(Sk), ptr(eig), ptr(eig_status), ptr(scratch[gi]),
                           int(scratch[gi].numel() * 8), int(sfx[2]), st)
            elif isinstance(sfx, int):
                self._call("skn_eigh_gen_large", count, ptr(db.n), ptr(db.hs_off), ptr(db.eoff), ptr(order_g),
                           ptr(Hk), ptr(Sk), ptr(eig), ptr(eig_status), ptr(counters[2 * gi:]), ptr(scratch[gi]),
                           int(scratch[gi].numel() * 8), max_n, sfx, st)
            else:
                self._call("skn_eigh_gen_batched" + sfx, count, ptr(db.n), ptr(db.hs_off), ptr(db.eoff),
                           ptr(order_g), ptr(Hk), ptr(Sk), ptr(eig), ptr(eig_status), ptr(counters[2 * gi:]),
                           max_n, st)

        if len(groups) == 1:
            launch(0, *groups[0], stream)
            return
        # one launch per group (in _groups' order) on forked streams
        main = torch.cuda.current_stream(self.device)
        fork = torch.cuda.Event()
        fork.record(main)
        joins = []
        for gi, g in enumerate(groups):
            st = self._side_streams(len(groups))[gi]
            st.wait_event(fork)
            with torch.cuda.stream(st):
                launch(gi, *g, st.cuda_stream)
            ev = torch.cuda.Event()
            ev.record(st)
            joins.append(ev)
        for ev in joins:
            main.wait_event(ev)

    def _side_streams(self, k):
        """k side streams for forked launches, cached per host thread and device (engines are
        created per batch by the server; creating streams per batch would cost more than the fork)."""
        pool = getattr(_SIDE, "pool", None)
        if pool is None:
            pool = _SIDE.pool = {}
        cur = pool.setdefault(self.device.index if self.device.index is not None else 0, [])
        while len(cur) < k:
            cur.append(torch.cuda.Stream(self.device))
        return cur

    def _groups(self, db):
        """[(launch shape suffix, the cluster size for the cluster path, or ("wide", n, real) for the
        device-wide path, device order, count, max_n)], cached on the batch.

        Empty when every problem takes the default single-CTA launch."""
        plan = db.plan
        key = (id(self.tuning), self.large_threshold, self.large_cluster, self.real_path, self.wide_threshold)
        cache = getattr(db, "_groups", None)
        if cache is not None and cache[0] == key:
            return cache[1]
        wide = route_wide(plan.prob_n, self.wide_threshold)[plan.order]
        csize = route_large(plan.prob_n, self.large_threshold, self.large_cluster)[plan.order]
        csize[wide] = 0
        large = (csize > 0) | wide
        out = []
        if wide.any():                       # one group per (n, real), largest first
            wn = plan.prob_n[plan.order[wide]]
            wr = (plan.prob_real[plan.order[wide]] if (self.real_path and plan.prob_real is not None)
                  else np.zeros(len(wn), dtype=bool))
            for n_, r_ in sorted({(int(a), bool(b)) for a, b in zip(wn, wr)}, reverse=True):
                sel = plan.order[wide][(wn == n_) & (wr == r_)]
                out.append((("wide", n_, int(r_)), sel, len(sel), n_))
        for c in sorted(set(csize[csize > 0].tolist()), reverse=True):    # one launch per cluster size
            sel = plan.order[csize == c]
            out.append((int(c), sel, len(sel), int(plan.prob_n[sel].max())))
        small_order = plan.order[~large]
        if len(small_order):
            tuning = self.tuning if self.tuning is not None else _default_tuning()
            shapes = [tuning.shape_for(int(n)) for n in plan.prob_n[small_order]]
            if self.real_path and plan.prob_real is not None:
                shapes = [("_real" + sh) if r else sh for sh, r in zip(shapes, plan.prob_real[small_order])]
            shapes = np.array(shapes, dtype=object)
            for sfx in dict.fromkeys(shapes.tolist()):
                sel = small_order[shapes == sfx]
                out.append((sfx, sel, len(sel), int(plan.prob_n[sel].max())))
        if len(out) == 1 and out[0][0] == "" and out[0][2] == len(plan.order):
            out = []     # the default launch over the batch's own order
        real = plan.prob_real if (self.real_path and plan.prob_real is not None) else np.zeros(len(plan.prob_n), bool)
        out = [out[i] for i in launch_order([g[1] for g in out], plan.prob_n, real)]
        out = [(sh, _i32(sel, self.device), cnt, mx) for sh, sel, cnt, mx in out]     # problem lists on the device
        db._groups = (key, out)
        return out

    def check_tables(self):
        """Raise if the last execute() needed a table the parameter set lacks (reads one device int)."""
        if int(self._status.item()) != 0:
            raise _lib.SknError("sk_blocks: a Slater-Koster table needed by this structure is missing")


class CapturedPath:
    """A batch whose geometry is fixed: the neighbour list is built once and kept on the
    device, and the rest of the path is captured in a CUDA graph.

    ``replay()`` re-runs phases, SK blocks, Bloch sums, eigensolve, Fermi/gap
    and DOS with no host work; it reads the tables from the ``TableSet``
    buffers, so writing new parameter values into ``tables.tab_H`` /
    ``tab_S`` in place (``refresh_tables``) and replaying evaluates the new
    parameters.  Outputs live in ``self.result`` (fixed addresses).
    """

    def __init__(self, engine: "Engine", db: DeviceBatch, **tail_kw):
        self.engine = engine
        self.db = db
        dev = engine.device
        self.bonds = engine.bonds(db)
        torch.cuda.synchronize(dev)
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):
            engine.tail(db, self.bonds, **tail_kw)          # warm-up outside the graph
        torch.cuda.current_stream(dev).wait_stream(side)
        torch.cuda.synchronize(dev)
        self.graph = torch.cuda.CUDAGraph()
        launches = engine.launches
        with torch.cuda.graph(self.graph, capture_error_mode="thread_local"):
            self.result = engine.tail(db, self.bonds, **tail_kw)
        self.kernels_per_replay = engine.launches - launches
        self.graph.replay()              # the capture itself runs nothing; fill the outputs once
        torch.cuda.synchronize(dev)
        engine.check_tables()

    def replay(self) -> "BatchResult":
        self.graph.replay()
        self.engine.launches += self.kernels_per_replay
        return self.result

    def refresh_tables(self, tables: "TableSet"):
        """Copy new table values into the captured buffers (same packing)."""
        T = self.engine.tables
        T.tab_H.copy_(tables.tab_H)
        T.tab_S.copy_(tables.tab_S)


class _nullctx:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def C_stream(st: torch.cuda.Stream):
    return st.cuda_stream
