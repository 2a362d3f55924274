"""DFTB+ Slater-Koster files (.skf) as model parameters.

The reference documents the skf format and keeps the column orders for it
(``Skf._sorter`` / ``_sorter_e``, slakonet/skf.py:24-115) but has no reader.
This module reads and writes the v1.0 format ("Format of the v1.0
Slater-Koster Files", dftb.org):

  simple (s, p, d)                     extended (s, p, d, f; first line "@")
  gridDist nGridPoints                 gridDist nGridPoints
  Ed Ep Es SPE Ud Up Us fd fp fs       Ef Ed Ep Es SPE Uf Ud Up Us ff fd fp fs   (A-A files only)
  mass c2..c9 rcut d1..d10             mass c2..c9 rcut d1..d10
  nGridPoints rows of 20 numbers       nGridPoints rows of 40 numbers
  [Spline section]                     [Spline section]

Each row holds the Hamiltonian then the overlap integrals at r = i * gridDist
(i = 1..nGridPoints), in the order

  dd0 dd1 dd2 pd0 pd1 pp0 pp1 sd0 sp0 ss0                                (simple)
  ff0 ff1 ff2 ff3 df0 df1 df2 dd0 dd1 dd2 pf0 pf1 pd0 pd1 pp0 pp1 sf0 sd0 sp0 ss0   (extended)

where "pd1" is the pi integral with the p orbital on the file's first atom
and the d orbital on the second.  Numbers may be separated by commas and may
use the "N*value" repetition shorthand and Fortran "D" exponents.

``read_skf`` returns the per-(l1, l2) integral tables in the model's layout
(``[l1 + 1, n_grid]``, rows sigma, pi, delta, phi); ``write_skf`` writes them
back; ``MultiElementSkfParameterOptimizer.from_skf_files`` builds a model from
a set of files.
"""
from __future__ import annotations

import os
import re
from typing import Dict, Optional, Tuple

import numpy as np

L = "spdf"
SIMPLE = ["dd0", "dd1", "dd2", "pd0", "pd1", "pp0", "pp1", "sd0", "sp0", "ss0"]
EXTENDED = ["ff0", "ff1", "ff2", "ff3", "df0", "df1", "df2", "dd0", "dd1", "dd2", "pf0", "pf1", "pd0", "pd1",
            "pp0", "pp1", "sf0", "sd0", "sp0", "ss0"]


def _numbers(line: str):
    out = []
    for tok in re.split(r"[\s,]+", line.strip()):
        if not tok:
            continue
        tok = tok.replace("D", "E").replace("d", "e")
        if "*" in tok:
            cnt, val = tok.split("*", 1)
            out.extend([float(val)] * int(cnt))
        else:
            out.append(float(tok))
    return out


def _tables(cols: np.ndarray, names, lmax: int) -> Dict[Tuple[int, int], np.ndarray]:
    idx = {nm: i for i, nm in enumerate(names)}
    out = {}
    for l1 in range(lmax + 1):
        for l2 in range(l1, lmax + 1):
            out[(l1, l2)] = np.stack([cols[:, idx[f"{L[l1]}{L[l2]}{m}"]] for m in range(l1 + 1)])
    return out


def read_skf(source: str, homonuclear: bool) -> dict:
    """Parse one skf file (a path, or the file's text).  ``homonuclear``: the file is A-A
    and carries the atomic line.  Returns grid_step, n_grid, H / S {(l1, l2): [l1+1, n]}
    (l1 <= l2; l1 on the first atom), atomic data (on_sites, hubbard_us, occupations by
    ascending l, spe, mass) for A-A files, mass, the repulsive polynomial and spline."""
    text = open(source).read() if os.path.exists(source) else source
    lines = [ln for ln in text.splitlines() if ln.strip()]
    extended = lines[0].lstrip().startswith("@")
    if extended:
        lines = lines[1:]
    head = _numbers(lines[0])
    step, n = float(head[0]), int(head[1])
    i = 1
    atomic = None
    if homonuclear:
        v = _numbers(lines[i])
        i += 1
        nl = 4 if extended else 3
        on = v[0:nl][::-1]                     # file: highest l first
        spe = v[nl]
        us = v[nl + 1: 2 * nl + 1][::-1]
        occ = v[2 * nl + 1: 3 * nl + 1][::-1]
        atomic = {"on_sites": on, "hubbard_us": us, "occupations": occ, "spe": spe}
    v = _numbers(lines[i])
    i += 1
    mass, r_poly = v[0], {"coef": v[1:9], "cutoff": v[9]}
    width = 40 if extended else 20
    rows = []
    while len(rows) < n:
        vals = _numbers(lines[i])
        i += 1
        if len(vals) != width:
            raise ValueError(f"skf row {len(rows) + 1} has {len(vals)} numbers, expected {width}")
        rows.append(vals)
    table = np.asarray(rows, dtype=np.float64)
    names = EXTENDED if extended else SIMPLE
    lmax = 3 if extended else 2
    half = width // 2
    H = _tables(table[:, :half], names, lmax)
    S = _tables(table[:, half:], names, lmax)
    r_spline = None
    rest = lines[i:]
    for j, ln in enumerate(rest):
        if ln.strip().lower().startswith("spline"):
            hdr = _numbers(rest[j + 1])
            nint, cut = int(hdr[0]), hdr[1]
            exp_coef = _numbers(rest[j + 2])
            seg = [_numbers(rest[j + 3 + q]) for q in range(nint)]
            r_spline = {"cutoff": cut, "exp_coef": exp_coef, "segments": seg}
            break
    if atomic is not None:
        atomic["mass"] = mass
    return {"grid_step": step, "n_grid": n, "H": H, "S": S, "atomic": atomic, "mass": mass,
            "r_poly": r_poly, "r_spline": r_spline, "extended": extended}


def write_skf(path: str, H: Dict[Tuple[int, int], np.ndarray], S: Dict[Tuple[int, int], np.ndarray],
              grid_step: float, atomic: Optional[dict] = None, mass: float = 0.0, extended: Optional[bool] = None):
    """Write integral tables in the v1.0 format (the inverse of ``read_skf``; integrals not
    given are written as zero, the repulsive polynomial as zeros with cutoff 1)."""
    lmax = max(max(k) for k in H)
    extended = lmax >= 3 if extended is None else extended
    names = EXTENDED if extended else SIMPLE
    n = next(iter(H.values())).shape[1]

    def cols(T):
        out = np.zeros((n, len(names)))
        for q, nm in enumerate(names):
            key = (L.index(nm[0]), L.index(nm[1]))
            if key in T:
                out[:, q] = np.asarray(T[key], dtype=np.float64)[int(nm[2])]
        return out

    table = np.concatenate([cols(H), cols(S)], 1)
    f = lambda x: repr(float(x))   # noqa: E731  shortest exact decimal
    out = ["@ extended format" if extended else None, f"{f(grid_step)} {n}"]
    out = [ln for ln in out if ln is not None]
    if atomic is not None:
        nl = 4 if extended else 3
        pad = lambda a: list(a) + [0.0] * (nl - len(a))   # noqa: E731
        on, us, occ = pad(atomic["on_sites"]), pad(atomic.get("hubbard_us", [])), pad(atomic["occupations"])
        vals = on[::-1] + [atomic.get("spe", 0.0)] + us[::-1] + occ[::-1]
        out.append(" ".join(f(v) for v in vals))
        mass = atomic.get("mass", mass)
    out.append(" ".join(f(v) for v in [mass] + [0.0] * 8 + [1.0] + [0.0] * 10))
    out += [" ".join(f(v) for v in row) for row in table]
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")


def grid_from_step(step: float, n: int) -> np.ndarray:
    """Distances of the rows: i * gridDist, i = 1..n (the reference's grid also starts at h)."""
    return step * np.arange(1, n + 1, dtype=np.float64)
