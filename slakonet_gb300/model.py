"""Drop-in model API: ``MultiElementSkfParameterOptimizer.compute_multi_element_properties``.

Mirrors the reference's model object (slakonet/optim.py:139-1443): a
``ModuleDict`` ``skf_optimizers`` keyed ``"A-B"`` by element symbols, each a
``SkfParameterOptimizer`` with ``h_params`` / ``s_params`` ParameterDicts
keyed ``"l1-l2"`` holding FP64 tensors ``[l1+1, n_grid]``.  State-dict keys
are therefore the reference's ``skf_optimizers.A-B.h_params.l1-l2``.

``compute_multi_element_properties`` keeps the reference signature and
returns the same ``(properties, True)`` pair (slakonet/optim.py:949-1075,
slakonet/main.py:1657-1819); the numbers come from the CUDA path in
``engine.py``.  There is no CPU path: a non-CUDA device raises.
"""
from __future__ import annotations

import itertools
import operator
import os
import re

import types
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch
import torch.nn as nn

from . import engine as E
from .elements import SYMBOLS, symbol_to_z

H2E = 27.211


class Geometry:
    """Minimal periodic geometry with the reference's attribute layout.

    ``atomic_numbers [1, N]``, ``positions [1, N, 3]`` and ``cell [1, 3, 3]``
    in Bohr (rows of ``cell`` are lattice vectors), as ``slakonet.atoms.Geometry``
    (slakonet/atoms.py:573-700).  Any object with these attributes is accepted
    by ``compute_multi_element_properties``.
    """

    _LEN = {"bohr": 1.0, "angstrom": 1.0 / 0.529177249}

    def __init__(self, atomic_numbers, positions, cell=None, units: str = "bohr"):
        f = self._LEN[units.lower()]
        z = torch.as_tensor(atomic_numbers).reshape(1, -1)
        p = torch.as_tensor(positions, dtype=torch.float64).reshape(1, -1, 3) * f
        self.atomic_numbers = z
        self.positions = p
        self.cell = None if cell is None else torch.as_tensor(cell, dtype=torch.float64).reshape(1, 3, 3) * f
        self.is_periodic = cell is not None

    @property
    def n_atoms(self):
        return self.atomic_numbers.count_nonzero(-1)

    @property
    def chemical_symbols(self) -> list:
        """Chemical symbols per batch entry, as ``Geometry.chemical_symbols`` (slakonet/atoms.py:751-754)."""
        from .elements import SYMBOLS
        return [[SYMBOLS[int(z)] for z in row if int(z) != 0] for row in self.atomic_numbers.tolist()]


def _structure_from_geometry(geometry) -> dict:
    z = torch.as_tensor(geometry.atomic_numbers).detach().cpu().reshape(-1).numpy()
    pos = torch.as_tensor(geometry.positions).detach().cpu().reshape(-1, 3).numpy()
    cell = getattr(geometry, "cell", None)
    if cell is None:
        raise ValueError("a periodic geometry with a cell is required")
    cell = torch.as_tensor(cell).detach().cpu().reshape(3, 3).numpy()
    keep = z != 0
    return {"numbers": z[keep].astype(np.int64), "positions": pos[keep].astype(np.float64),
            "cell": cell.astype(np.float64)}


def mp_kpoints(mesh) -> np.ndarray:
    """Offset Monkhorst-Pack grid ``0.5/n + i/n`` (slakonet/atoms.py:394-446), x slowest."""
    n1, n2, n3 = (int(v) for v in np.asarray(mesh).reshape(-1)[:3])
    a = 0.5 / n1 + np.arange(n1) * (1.0 / n1)
    b = 0.5 / n2 + np.arange(n2) * (1.0 / n2)
    c = 0.5 / n3 + np.arange(n3) * (1.0 / n3)
    return np.stack(np.meshgrid(a, b, c, indexing="ij"), -1).reshape(-1, 3)


def reduce_time_reversal(kpoints, weights=None, tol: float = 1e-9):
    """Halve a k-point list by time reversal: ``(k_red, w_red, index)``.

    The real-space blocks H(T), S(T) are real, so H(-k) and S(-k) are the complex conjugates of H(k) and
    S(k), and the eigenvalues at -k equal those at k.  Of each pair {k, -k modulo reciprocal lattice
    vectors} found in the list, the first stays in ``k_red`` with the pair's weights summed; a k-point that
    is its own partner (2k integer: Gamma and zone-boundary points) or whose partner is absent stays with
    its own weight.  ``index[i]`` is the row of ``k_red`` whose eigenvalues are k-point i's, so
    ``eig_red[index]`` restores the full list's eigenvalues, and the reduced list with ``w_red`` gives the
    full list's Fermi level, gap and DOS (the same eigenvalues with the same total weight) for about half
    the eigensolves on Monkhorst-Pack and Gamma-centred grids.  The reference solves every k-point.  Partner
    eigenvalues agree to rounding (the partner's phases come from -k or from 1 - k, which round differently)."""
    k = np.asarray(kpoints, dtype=np.float64).reshape(-1, 3)
    nk = len(k)
    w = np.full(nk, 1.0 / max(nk, 1)) if weights is None else np.asarray(weights, dtype=np.float64).reshape(-1)
    if len(w) != nk:
        raise ValueError(f"{len(w)} weights for {nk} k-points")
    scale = 1.0 / tol
    period = int(round(scale))

    def key(v):
        q = np.mod(np.round(v * scale).astype(np.int64), period)
        return tuple(int(x) for x in q)
    first = {}
    for i in range(nk):
        first.setdefault(key(k[i]), []).append(i)
    index = np.full(nk, -1, np.int64)
    keep, wk = [], []
    for i in range(nk):
        if index[i] >= 0:
            continue
        index[i] = len(keep)
        keep.append(i)
        wsum = w[i]
        for j in first.get(key(-k[i]), []):
            if j != i and index[j] < 0:
                index[j] = index[i]
                wsum += w[j]
                break
        wk.append(wsum)
    return k[keep].copy(), np.array(wk, dtype=np.float64), index


def klines_kpoints(klines) -> np.ndarray:
    """Band-path points ``k1 + i (k2-k1)/(N-1)`` per segment (slakonet/atoms.py:448-502)."""
    kl = np.asarray(torch.as_tensor(klines).detach().cpu().numpy(), dtype=np.float64).reshape(-1, 7)
    pts = []
    for row in kl:
        n = int(row[6])
        d = row[3:6] - row[0:3]
        if n >= 1:
            with np.errstate(divide="ignore", invalid="ignore"):
                d = d / (row[6] - 1.0)
        pts.extend(row[0:3] + d * i for i in range(n))
    return np.array(pts, dtype=np.float64).reshape(-1, 3)


# Parameter values reach the device tables through MultiElementSkfParameterOptimizer.table_set,
# which repacks only when a parameter changed.  Changes are seen through the tensors' version
# counters (in-place updates under no_grad, optimizer steps, load_state_dict, apply_constraints)
# and, for the set of parameters itself, through this epoch, bumped whenever a parameter
# container or entry is replaced.  Assigning ``p.data`` directly bypasses both: call
# ``invalidate_tables()`` after doing so.
_PARAM_EPOCH = [0]


def _bump_epoch():
    _PARAM_EPOCH[0] += 1


class _TrackedParameterDict(nn.ParameterDict):
    def __setitem__(self, key, value):
        super().__setitem__(key, value)
        _bump_epoch()

    def __delitem__(self, key):
        super().__delitem__(key)
        _bump_epoch()


class _TrackedModuleDict(nn.ModuleDict):
    def __setitem__(self, key, module):
        super().__setitem__(key, module)
        _bump_epoch()

    def __delitem__(self, key):
        super().__delitem__(key)
        _bump_epoch()


class SkfParameterOptimizer(nn.Module):
    """Trainable tables of one element pair (slakonet/optim.py:1356-1443)."""

    def __init__(self, atom_pair: Sequence[int], h: Dict[str, torch.Tensor], s: Dict[str, torch.Tensor],
                 grid, atomic_data: Optional[dict] = None, hs_cutoff=None):
        super().__init__()
        self.h_params = _TrackedParameterDict({k: nn.Parameter(torch.as_tensor(v, dtype=torch.float64).clone())
                                          for k, v in h.items()})
        self.s_params = _TrackedParameterDict({k: nn.Parameter(torch.as_tensor(v, dtype=torch.float64).clone())
                                          for k, v in s.items()})
        self.original_h_params = {k: v.detach().clone() for k, v in self.h_params.items()}
        self.original_s_params = {k: v.detach().clone() for k, v in self.s_params.items()}
        self.atom_pair = [int(atom_pair[0]), int(atom_pair[1])]
        self.grid = [float(g) for g in np.asarray(grid).reshape(-1)]
        self.atomic_data = atomic_data
        self.hs_cutoff = hs_cutoff if hs_cutoff is not None else self.grid[-1]
        self.skf_dict = {"atom_pair": self.atom_pair, "grid": self.grid, "hs_cutoff": self.hs_cutoff,
                         "atomic": atomic_data is not None}
        if atomic_data is not None:
            self.skf_dict["atomic_data"] = atomic_data

    def __setattr__(self, name, value):
        super().__setattr__(name, value)
        if name in ("h_params", "s_params"):
            _bump_epoch()

    @property
    def grid_step(self) -> float:
        return self.grid[1] - self.grid[0]

    def constraint_bounds(self, c=(0.9, 0.7, 0.95, 0.9), device=None):
        """(parameters, lower, upper) of ``apply_constraints``: the same bounds as tensors, so a
        caller can clamp many pairs at once."""
        ps, lo, hi = [], [], []
        for key, p in self.h_params.items():
            o = self.original_h_params[key].to(device if device is not None else p.device)
            f = c[0] if key.split("-")[0] == key.split("-")[1] else c[1]
            ps.append(p)
            lo.append(o * f)
            hi.append(o * (1 + (1 - f)))
        for key, p in self.s_params.items():
            o = self.original_s_params[key].to(device if device is not None else p.device)
            ps.append(p)
            if key.split("-")[0] == key.split("-")[1]:
                lo.append(torch.maximum(o * c[2], torch.tensor(0.1, dtype=o.dtype, device=o.device)))
                hi.append(o * (1 + (1 - c[2])))
            else:
                lo.append(o * c[3])
                hi.append(o * (1 + (1 - c[3])))
        return ps, lo, hi

    def apply_constraints(self, c=(0.9, 0.7, 0.95, 0.9)):
        """Clamp parameters to a band around their initial values (slakonet/optim.py:1392-1434)."""
        # same bounds as the reference, applied in place (which the table cache sees)
        with torch.no_grad():
            for key, p in self.h_params.items():
                o = self.original_h_params[key].to(p.device)
                f = c[0] if key.split("-")[0] == key.split("-")[1] else c[1]
                p.copy_(torch.clamp(p, o * f, o * (1 + (1 - f))))
            for key, p in self.s_params.items():
                o = self.original_s_params[key].to(p.device)
                if key.split("-")[0] == key.split("-")[1]:
                    p.copy_(torch.clamp(p, torch.maximum(o * c[2], torch.tensor(0.1, dtype=o.dtype, device=o.device)),
                                        o * (1 + (1 - c[2]))))
                else:
                    p.copy_(torch.clamp(p, o * c[3], o * (1 + (1 - c[3]))))


class MultiElementSkfParameterOptimizer(nn.Module):
    """Model object with the reference's parameter layout and property API."""

    def __init__(self):
        super().__init__()
        self.skf_optimizers = _TrackedModuleDict()
        self.atomic_num_to_symbol = {z: SYMBOLS[z] for z in range(1, len(SYMBOLS))}
        self._table_cache = None
        self.__dict__["_invalidations"] = 0

    # ------------------------------------------------------------ building
    @classmethod
    def from_tables(cls, tables: dict) -> "MultiElementSkfParameterOptimizer":
        """From ``synthetic.make_tables`` output (grid, per-pair H/S, element data)."""
        m = cls()
        for (za, zb), pair in sorted(tables["pairs"].items()):
            h = {f"{l1}-{l2}": v for (l1, l2), v in pair["H"].items()}
            s = {f"{l1}-{l2}": v for (l1, l2), v in pair["S"].items()}
            atomic = None
            if za == zb:
                el = tables["elements"][za]
                atomic = {"on_sites": [float(x) for x in el["on_sites"]],
                          "hubbard_us": [0.0] * len(el["on_sites"]), "mass": 1.0,
                          "occupations": [float(x) for x in el["occupations"]]}
            m.skf_optimizers[f"{SYMBOLS[za]}-{SYMBOLS[zb]}"] = SkfParameterOptimizer(
                (za, zb), h, s, tables["grid"], atomic)
        return m

    @classmethod
    def from_skf_files(cls, files) -> "MultiElementSkfParameterOptimizer":
        """From DFTB+ Slater-Koster files: a directory of ``A-B.skf`` files, or a dict
        ``{(za, zb) or "A-B": path}``.  Every ordered pair needs its file (A-B and B-A), and
        every element its A-A file (on-site energies, occupations).  See ``slakonet_gb300.skf``."""
        from . import skf as SKF
        if isinstance(files, (str, os.PathLike)):
            found = {}
            for name in sorted(os.listdir(files)):
                m_ = re.fullmatch(r"([A-Z][a-z]?)-([A-Z][a-z]?)\.skf", name)
                if m_:
                    found[(SYMBOLS.index(m_.group(1)), SYMBOLS.index(m_.group(2)))] = os.path.join(files, name)
            files = found
        m = cls()
        for key, path in sorted(((k if isinstance(k, tuple) else tuple(SYMBOLS.index(x) for x in k.split("-"))), v)
                                for k, v in files.items()):
            za, zb = int(key[0]), int(key[1])
            d = SKF.read_skf(path, homonuclear=(za == zb))
            h = {f"{l1}-{l2}": v for (l1, l2), v in d["H"].items()}
            s_ = {f"{l1}-{l2}": v for (l1, l2), v in d["S"].items()}
            atomic = None
            if za == zb:
                a = d["atomic"]
                atomic = {"on_sites": [float(x) for x in a["on_sites"]],
                          "hubbard_us": [float(x) for x in a["hubbard_us"]], "mass": float(a["mass"]),
                          "occupations": [float(x) for x in a["occupations"]]}
            grid = SKF.grid_from_step(d["grid_step"], d["n_grid"])
            m.skf_optimizers[f"{SYMBOLS[za]}-{SYMBOLS[zb]}"] = SkfParameterOptimizer((za, zb), h, s_, grid, atomic)
        return m

    def write_skf_files(self, directory: str):
        """Write every pair's current parameters as ``A-B.skf`` (DFTB+ v1.0 format)."""
        from . import skf as SKF
        os.makedirs(directory, exist_ok=True)
        for key, opt in self.skf_optimizers.items():
            H = {tuple(int(x) for x in k.split("-")): v.detach().cpu().numpy() for k, v in opt.h_params.items()}
            S = {tuple(int(x) for x in k.split("-")): v.detach().cpu().numpy() for k, v in opt.s_params.items()}
            SKF.write_skf(os.path.join(directory, f"{key}.skf"), H, S, opt.grid_step, opt.atomic_data)

    @classmethod
    def load_ultra_compact(cls, path: str) -> "MultiElementSkfParameterOptimizer":
        """Read the reference's ultra-compact checkpoint (slakonet/optim.py:528-625).

        The file holds ``metadata`` (``available_pairs``), ``skf_metadata``
        (grid, atomic data per pair) and ``trained_parameters`` (a state dict
        with ``skf_optimizers.A-B.{h,s}_params.l1-l2`` keys).
        """
        data = torch.load(path, map_location="cpu", weights_only=False)
        meta, sd, skm = data["metadata"], data["trained_parameters"], data["skf_metadata"]
        m = cls()
        m.skf_directory = meta.get("skf_directory")
        for pk in meta["available_pairs"]:
            h, s = {}, {}
            for key, v in sd.items():
                if key.startswith(f"skf_optimizers.{pk}.h_params."):
                    h[key.split(".")[-1]] = v
                elif key.startswith(f"skf_optimizers.{pk}.s_params."):
                    s[key.split(".")[-1]] = v
            md = skm[pk]
            opt = SkfParameterOptimizer(md["atom_pair"], h, s, md["grid"], md.get("atomic_data"), md.get("hs_cutoff"))
            # the rest of the pair's metadata travels unchanged to save_ultra_compact
            opt.skf_dict.update({k: v for k, v in md.items()
                                 if k not in ("hamiltonian", "overlap", "atom_pair", "grid", "hs_cutoff")})
            m.skf_optimizers[pk] = opt
        m.load_state_dict(sd, strict=False)
        return m

    def save_ultra_compact(self, path) -> str:
        """Write the reference's ultra-compact checkpoint (slakonet/optim.py:485-519), the file
        ``load_ultra_compact`` reads here and in the reference: ``metadata`` (pairs and elements),
        ``trained_parameters`` (the state dict: after fitting, the fitted values) and ``skf_metadata`` (each
        pair's grid, cutoff and atomic data, without the tables the state dict already holds).  Only
        tensors, numbers, strings, lists and dicts are stored, so ``torch.load(..., weights_only=True)`` --
        what the reference's loader does under current PyTorch -- reads it.  The suffix becomes ``.pt``, as in
        the reference; returns the path written."""
        root, ext = os.path.splitext(os.fspath(path))
        out = root + ".pt"
        os.makedirs(os.path.dirname(os.path.abspath(out)), exist_ok=True)

        def plain(v):
            if isinstance(v, np.ndarray):
                return torch.as_tensor(v.copy())
            if isinstance(v, np.generic):
                return v.item()
            if isinstance(v, torch.Tensor):
                return v.detach().cpu().clone()
            if isinstance(v, dict):
                return {k: plain(x) for k, x in v.items()}
            if isinstance(v, (list, tuple)):
                return [plain(x) for x in v]
            return v
        pairs = list(self.skf_optimizers.keys())
        elems = sorted({int(z) for opt in self.skf_optimizers.values() for z in opt.atom_pair})
        data = {
            "metadata": {"skf_directory": getattr(self, "skf_directory", None), "elements_in_system": elems,
                         "element_pairs": [[int(z) for z in opt.atom_pair] for opt in self.skf_optimizers.values()],
                         "available_pairs": pairs, "class_name": "MultiElementSkfParameterOptimizer",
                         "ultra_compact": True},
            "trained_parameters": {k: v.detach().cpu().clone() for k, v in self.state_dict().items()},
            "skf_metadata": {pk: plain({k: v for k, v in opt.skf_dict.items() if k not in ("hamiltonian", "overlap")})
                             for pk, opt in self.skf_optimizers.items()},
        }
        torch.save(data, out)
        return out

    def get_updated_skfs(self):
        """Per-pair dicts of live parameters (the data ``Skf.from_dict`` would wrap)."""
        out = {}
        for key, opt in self.skf_optimizers.items():
            d = dict(opt.skf_dict)
            d["hamiltonian"] = dict(opt.h_params.items())
            d["overlap"] = dict(opt.s_params.items())
            out[key] = d
        return out

    def apply_constraints(self, c=(0.9, 0.7, 0.95, 0.9)):
        """Every pair's ``apply_constraints`` (slakonet/optim.py:1392-1434) at once: the bounds are
        built on the parameters' device the first time and kept, and the clamp
        min(max(p, lower), upper) -- exactly torch.clamp, including its behaviour when lower > upper
        for negative amplitudes -- runs as two fused in-place operations over all parameters."""
        plist = self._param_list()
        key = (_PARAM_EPOCH[0], tuple(c), tuple(sorted({str(p.device) for p in plist})))
        cached = self.__dict__.get("_bounds")
        if cached is None or cached[0] != key:
            ps, lo, hi = [], [], []
            for opt in self.skf_optimizers.values():
                a, b, d = opt.constraint_bounds(c)
                ps += a
                lo += b
                hi += d
            cached = (key, ps, lo, hi)
            self.__dict__["_bounds"] = cached
        _, ps, lo, hi = cached
        if not ps:
            return
        with torch.no_grad():
            torch._foreach_maximum_(ps, lo)
            torch._foreach_minimum_(ps, hi)

    # ------------------------------------------------------------- feeding
    def __setattr__(self, name, value):
        super().__setattr__(name, value)
        if name == "skf_optimizers":
            _bump_epoch()

    def _param_list(self):
        cached = self.__dict__.get("_plist")
        if cached is None or cached[0] != _PARAM_EPOCH[0]:
            plist = [p for opt in self.skf_optimizers.values()
                     for p in itertools.chain(opt.h_params.values(), opt.s_params.values())]
            cached = (_PARAM_EPOCH[0], plist)
            self.__dict__["_plist"] = cached
        return cached[1]

    def _param_signature(self, device):
        """(layout key, value key): the layout changes with the parameter set, the value key with any
        in-place update (version counters only grow, so their sum changes whenever any of them does)."""
        plist = self._param_list()
        return (str(device), _PARAM_EPOCH[0], self._invalidations), sum(map(operator.attrgetter("_version"), plist))

    def invalidate_tables(self):
        """Repack the device tables on the next call (needed only after assigning ``p.data`` directly)."""
        self.__dict__["_invalidations"] = self._invalidations + 1

    def table_set(self, shell_dict: Dict[int, List[int]], device, species: Optional[Sequence[int]] = None):
        """Packed device tables for ``species`` (all elements of the model by default), cached."""
        species = sorted(set(int(z) for z in (species if species is not None else self._elements())))
        layout, values = self._param_signature(device)
        key = (layout, tuple(species), tuple((z, tuple(shell_dict[z])) for z in species))
        if self._table_cache is not None and self._table_cache[0] == key:
            if self._table_cache[2] == values:
                return self._table_cache[1]
            ts = self._table_cache[1].with_values()      # same layout, new values: repack values only
            if ts is not None:
                self._table_cache = (key, ts, values)
                return ts
        h, s, steps, onsite, occ = {}, {}, {}, {}, {}
        sset = set(species)
        for key_, opt in self.skf_optimizers.items():
            za, zb = opt.atom_pair
            if za not in sset or zb not in sset:
                continue
            h[(za, zb)] = {tuple(int(x) for x in k.split("-")): v for k, v in opt.h_params.items()}
            s[(za, zb)] = {tuple(int(x) for x in k.split("-")): v for k, v in opt.s_params.items()}
            steps[(za, zb)] = opt.grid_step
            if za == zb and opt.atomic_data is not None:
                onsite[za] = np.asarray(opt.atomic_data["on_sites"], dtype=np.float64)
                occ[za] = np.asarray(opt.atomic_data["occupations"], dtype=np.float64)
        missing = [z for z in species if z not in onsite]
        if missing:
            raise ValueError(f"no homonuclear parameters (on-site energies) for Z={missing}")
        ts = E.TableSet(species, shell_dict, h, s, steps, onsite, occ, device)
        self._table_cache = (key, ts, values)
        return ts

    def _elements(self):
        zs = set()
        for opt in self.skf_optimizers.values():
            zs.update(opt.atom_pair)
        return zs

    # ----------------------------------------------------------- properties
    def compute_properties_batch(self, structures: Sequence[dict], shell_dict=None, device=None,
                                 dos_range=(-10.0, 10.0), dos_points: int = 5000, dos_sigma: float = 0.1,
                                 dos_window: float = 0.0, cutoff: float = E.CUTOFF_BOHR, engine=None,
                                 with_eigenvectors: bool = False):
        """Batched path: many structures (each with its own k-points) in one launch sequence.

        Each structure is a dict with ``numbers``, ``positions`` and ``cell``
        (Bohr) and ``kpoints`` ([nk, 3] fractional; optional ``weights``).
        Returns the ``BatchResult`` (device tensors).
        """
        device = torch.device(device if device is not None else "cuda")
        shell_dict = shell_dict if shell_dict is not None else _default_shell_dict()
        zs = sorted(set(int(z) for st in structures for z in np.asarray(st["numbers"]).reshape(-1)))
        ts = self.table_set(shell_dict, device, zs)
        eng = engine or E.Engine(ts, cutoff)
        plan = E.plan_batch(structures, ts, cutoff)
        res = eng.run(plan, dos_range, dos_points, dos_sigma, dos_window, vectors=with_eigenvectors)
        eng.check_tables()
        return res

    def compute_multi_element_properties(self, geometry=None, shell_dict=None, kpoints=None, klines=None,
                                         phonons=False, get_fermi=False, get_energy=False, get_forces=False,
                                         get_bulk_mod=False, device=None, with_eigenvectors=False):
        """Reference signature (slakonet/optim.py:949-962); returns ``(properties, True)``."""
        if phonons or get_bulk_mod:
            raise NotImplementedError("phonons and the bulk modulus are outside this path")
        if device is None:
            device = "cuda"
        device = torch.device(device)
        shell_dict = shell_dict if shell_dict is not None else _default_shell_dict()
        st = _structure_from_geometry(geometry)
        if klines is not None:
            k = klines_kpoints(klines)
        elif kpoints is not None:
            k = mp_kpoints(torch.as_tensor(kpoints).detach().cpu().numpy())
        else:
            k = mp_kpoints([1, 1, 1])
        st["kpoints"] = k
        st["weights"] = np.full(len(k), 1.0 / len(k))
        res = self.compute_properties_batch([st], shell_dict, device, with_eigenvectors=with_eigenvectors)
        props = properties_dict(res, 0, get_fermi=get_fermi)
        if "calc" in props:
            props["calc"].geometry = geometry     # as the reference's calculator (SimpleDftb.geometry)
        if get_energy:      # slakonet/optim.py:1066-1068
            props["total_energy"] = res.stats[0, E.STAT["band_energy_ha"]]
        if get_forces:      # slakonet/optim.py:1069-1071
            props["forces"] = self.finite_difference_forces(st, shell_dict, device)
        return props, True

    def finite_difference_forces(self, structure: dict, shell_dict=None, device=None, delta: float = 1e-2,
                                 mesh=(5, 5, 5)) -> torch.Tensor:
        """Forces as ``SimpleDftb._compute_forces_finite_diff`` (slakonet/main.py:198-281):
        F_ij = -(E(+) - E(-)) / (2 delta), E the plain sum of every eigenvalue on a ``mesh``
        Monkhorst-Pack grid, atom i displaced by +-delta Bohr along axis j.  The reference
        runs the 6N displaced structures one after another; here all of them (6N x nk
        problems) go through the path as one batch.  Returns [1, N, 3] (Hartree/Bohr)."""
        device = torch.device(device if device is not None else "cuda")
        pos = np.asarray(structure["positions"], dtype=np.float64).reshape(-1, 3)
        k = mp_kpoints(mesh)
        displaced = []
        for i in range(len(pos)):
            for j in range(3):
                for sgn in (1.0, -1.0):
                    p = pos.copy()
                    p[i, j] += sgn * delta
                    displaced.append({"numbers": structure["numbers"], "positions": p, "cell": structure["cell"],
                                      "kpoints": k})
        res = self.compute_properties_batch(displaced, shell_dict, device, dos_points=1)
        per = int(res.plan.nk[0]) * int(res.plan.nb[0])
        sums = res.eig[: len(displaced) * per].view(len(displaced), per).sum(1).view(len(pos), 3, 2)
        return (-(sums[..., 0] - sums[..., 1]) / (2.0 * delta)).unsqueeze(0)


def _default_shell_dict():
    from .synthetic import default_shell_dict
    return default_shell_dict()


def properties_dict(res: "E.BatchResult", s: int, get_fermi: bool = False) -> dict:
    """The reference's properties dict for structure ``s`` of a batch result."""
    plan = res.plan
    st = res.stats[s].detach().cpu().numpy()
    I = E.STAT
    dev = res.eig.device
    eig = res.eigenvalues(s).unsqueeze(0)
    metal_or_fallback = st[I["metal"]] > 0 or st[I["fallback"]] > 0
    gap_t = torch.tensor(float(st[I["gap_ev"]]), dtype=torch.float64, device="cpu" if metal_or_fallback else dev)
    mdg = st[I["min_dgap"]]
    dos = res.dos[s]
    props = {
        "fermi_energy_eV": float(st[I["fermi_ev"]]),
        "fermi_energy_Ha": float(st[I["mu_ha"]]),
        "band_gap_eV": gap_t,
        "vbm_eV": float(st[I["vbm_ev"]]),
        "cbm_eV": float(st[I["cbm_ev"]]),
        "is_direct_gap": bool(st[I["direct"]] > 0),
        "vbm_kpoint": int(st[I["vbm_k"]]),
        "cbm_kpoint": int(st[I["cbm_k"]]),
        "valence_band_width_eV": float(st[I["vwidth"]]),
        "conduction_band_width_eV": float(st[I["cwidth"]]),
        "minimum_direct_gap_eV": None if np.isnan(mdg) else float(mdg),
        "is_direct_semiconductor": torch.tensor(bool(st[I["direct_semi"]] > 0)),
        "nkpoints": int(plan.nk[s]),
        "nbands": int(plan.nb[s]),
        "nelectrons": int(plan.nelec[s]),
        "dos_at_fermi": float(st[I["dos_fermi"]]),
        "dos_gap_center_eV": float(st[I["dos_gapc"]]),
        "dos_total_states": float(st[I["dos_total"]]),
        "dos_at_fermi_tensor": res.stats[s, I["dos_fermi"]],
        "dos_gap_center_tensor": res.stats[s, I["dos_gapc"]],
        "dos_total_states_tensor": res.stats[s, I["dos_total"]],
        "dos_energy_grid_tensor": res.dos_grid,
        "dos_values_tensor": dos,
        "fermi_converged": bool(st[I["converged"]] > 0),
    }
    k0 = int(plan.k_ptr[s])
    nk = int(plan.nk[s])
    calc = types.SimpleNamespace(
        eigenvalue=eig,
        k_weights=torch.as_tensor(plan.kweights[k0:k0 + nk]).unsqueeze(0),
        kpoints=torch.as_tensor(plan.kpoints[k0:k0 + nk]).unsqueeze(0),
        nelectron=torch.tensor([plan.nelec[s]]),
    )
    if res.vec is not None:   # reference layout [1, n (component), n (band), nk]
        calc.eigenvectors = res.eigenvectors(s).permute(1, 2, 0).unsqueeze(0)
    if get_fermi:
        props["efermi"] = (res.mu[s] * H2E).reshape(1, 1, 1)
        props["bandgap"] = res.stats[s, I["bandgap_ev"]].reshape(1)
        props["calc"] = calc
    props["eigenvalues"] = eig
    return props
