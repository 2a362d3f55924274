"""Seeded synthetic Slater-Koster parameter sets and structures.

The reference's pretrained parameters are a network download and its test
structures are missing, so every workload here is synthetic.  This module
is the single definition of those inputs; the fixtures, the tests and
``bench.py`` all draw from it, so the same seed always gives the same
numbers.

Parameter layout follows the reference's ``Skf`` container
(slakonet/skf.py:152-199): per ordered element pair ``(A, B)`` a dict of
Hamiltonian and overlap tables keyed ``(l1, l2)`` with ``l1 <= l2``, each an
array ``[l1 + 1, n_grid]`` (sigma, pi, delta, phi rows) on the grid
``h * (1 .. n_grid)`` in Bohr, integrals in Hartree.  A table ``(A, B)``
holds every key with ``l1`` a shell of ``A`` and ``l2`` a shell of ``B``.

Integral model: ``A * exp(-b r)`` with ``A ~ U(-5, 5) eV`` for H and
``U(-0.5, 0.5)`` for S, ``b ~ U(0.5, 1.5) / Angstrom``.  On-site energies:
s ~ U(-12, -6), p ~ U(-6, 0), d ~ U(-2, 4), f ~ U(-4, 2) eV.
Occupations: neutral valence count (electrons outside the last noble-gas
core, with a filled d10 shell counted as core for the p-block elements the
default shell map treats as s,p only), capped at ``2 * n_orbitals``, filled
s, p, d, f in order.
"""
from __future__ import annotations

import math
from typing import Dict, Iterable, List, Tuple

import numpy as np

BOHR_ANGSTROM = 0.529177249          # slakonet/units.py:63
ANGSTROM_TO_BOHR = 1.0 / BOHR_ANGSTROM
EV_PER_HARTREE_SYNTH = 27.2113845    # conversion used only to build synthetic tables
H2E = 27.211                          # eV per Hartree on the properties path (slakonet/main.py:34)

GRID_STEP = 0.02                       # Bohr
GRID_MAX_ANGSTROM = 7.0


def default_shell_dict() -> Dict[int, List[int]]:
    """Angular momenta per element, as ``generate_shell_dict_upto_Z65`` (slakonet/main.py:37-59)."""
    out = {}
    for z in range(1, 100):
        if z <= 2:
            out[z] = [0]
        elif z <= 20:
            out[z] = [0, 1]
        elif z <= 30:
            out[z] = [0, 1, 2]
        elif z <= 36:
            out[z] = [0, 1]
        elif z <= 48:
            out[z] = [0, 1, 2]
        elif z <= 54:
            out[z] = [0, 1]
        elif z <= 57:
            out[z] = [0, 1, 2]
        else:
            out[z] = [0, 1, 2, 3]
    return out


def grid_points(step: float = GRID_STEP, rmax_angstrom: float = GRID_MAX_ANGSTROM) -> np.ndarray:
    n = int(math.floor(rmax_angstrom * ANGSTROM_TO_BOHR / step + 1e-9))
    return step * np.arange(1, n + 1, dtype=np.float64)


_NOBLE = [0, 2, 10, 18, 36, 54, 86]


def valence_electrons(z: int, shells: List[int]) -> int:
    core = max(c for c in _NOBLE if c < z) if z > 2 else 0
    if 31 <= z <= 36:
        core = 28
    elif 49 <= z <= 54:
        core = 46
    nval = z - core
    norb = sum(2 * l + 1 for l in shells)
    return int(min(nval, 2 * norb))


def shell_occupations(z: int, shells: List[int]) -> List[float]:
    left = valence_electrons(z, shells)
    occ = []
    for l in sorted(shells):
        cap = 2 * (2 * l + 1)
        take = min(cap, left)
        occ.append(float(take))
        left -= take
    return occ


_ONSITE_EV = {0: (-12.0, -6.0), 1: (-6.0, 0.0), 2: (-2.0, 4.0), 3: (-4.0, 2.0)}


def make_tables(elements: Iterable[int], shell_dict: Dict[int, List[int]] | None = None,
                seed: int = 0, step: float = GRID_STEP,
                rmax_angstrom: float = GRID_MAX_ANGSTROM) -> dict:
    """Synthetic tables for every ordered pair of ``elements``.

    Draw order (numpy PCG64, ``seed``): elements ascending, each element's
    on-site energies s, p, d, f; then ordered pairs ``(A, B)`` ascending, for
    each key ``(l1, l2)`` ascending and each bond order, H amplitude, H decay,
    S amplitude, S decay.
    """
    shell_dict = default_shell_dict() if shell_dict is None else shell_dict
    els = sorted(set(int(z) for z in elements))
    rng = np.random.default_rng(seed)
    grid = grid_points(step, rmax_angstrom)
    r = grid
    out_el = {}
    for z in els:
        shells = list(shell_dict[z])
        lmax = max(shells)
        on = [rng.uniform(*_ONSITE_EV[l]) / EV_PER_HARTREE_SYNTH for l in range(4)]
        out_el[z] = {
            "shells": shells,
            "on_sites": np.array(on[: lmax + 1], dtype=np.float64),
            "occupations": np.array(shell_occupations(z, shells), dtype=np.float64),
        }
    pairs = {}
    for za in els:
        for zb in els:
            la_set = sorted(set(shell_dict[za]))
            lb_set = sorted(set(shell_dict[zb]))
            keys = sorted({(l1, l2) for l1 in la_set for l2 in lb_set if l1 <= l2})
            H, S = {}, {}
            for (l1, l2) in keys:
                m = l1 + 1
                h = np.empty((m, len(grid)))
                s = np.empty((m, len(grid)))
                for bo in range(m):
                    ah = rng.uniform(-5.0, 5.0) / EV_PER_HARTREE_SYNTH
                    bh = rng.uniform(0.5, 1.5) * BOHR_ANGSTROM
                    as_ = rng.uniform(-0.5, 0.5)
                    bs = rng.uniform(0.5, 1.5) * BOHR_ANGSTROM
                    h[bo] = ah * np.exp(-bh * r)
                    s[bo] = as_ * np.exp(-bs * r)
                H[(l1, l2)] = h
                S[(l1, l2)] = s
            pairs[(za, zb)] = {"H": H, "S": S}
    return {"grid": grid, "step": float(step), "elements": out_el, "pairs": pairs,
            "shell_dict": {z: list(shell_dict[z]) for z in els}}


def perturb_tables(tables: dict, rel_sigma: float, seed: int) -> dict:
    """Copy of ``tables`` with every H and S amplitude scaled by ``1 + N(0, rel_sigma)``."""
    rng = np.random.default_rng(seed)
    out = {k: v for k, v in tables.items() if k != "pairs"}
    out["pairs"] = {}
    for pk in sorted(tables["pairs"]):
        pair = tables["pairs"][pk]
        npair = {"H": {}, "S": {}}
        for kind in ("H", "S"):
            for key in sorted(pair[kind]):
                t = pair[kind][key]
                f = 1.0 + rel_sigma * rng.standard_normal((t.shape[0], 1))
                npair[kind][key] = t * f
        out["pairs"][pk] = npair
    return out


# ---------------------------------------------------------------- structures

def diamond_si(a_angstrom: float = 5.43) -> dict:
    """2-atom diamond-cubic Si: fcc cell, atoms at (0,0,0) and (1/4,1/4,1/4) a."""
    a = a_angstrom * ANGSTROM_TO_BOHR
    cell = 0.5 * a * np.array([[0.0, 1.0, 1.0], [1.0, 0.0, 1.0], [1.0, 1.0, 0.0]])
    pos = np.array([[0.0, 0.0, 0.0], [0.25 * a, 0.25 * a, 0.25 * a]])
    return {"numbers": np.array([14, 14]), "positions": pos, "cell": cell}


def zincblende_supercell(reps: int = 5, a_angstrom: float = 5.65, jitter_angstrom: float = 0.05,
                         z1: int = 31, z2: int = 33, seed: int = 0) -> dict:
    """``reps^3`` conventional 8-atom zincblende cells with Gaussian site jitter."""
    rng = np.random.default_rng(seed)
    a = a_angstrom * ANGSTROM_TO_BOHR
    fcc = np.array([[0, 0, 0], [0, 0.5, 0.5], [0.5, 0, 0.5], [0.5, 0.5, 0]])
    basis = np.concatenate([fcc, fcc + 0.25])
    species = [z1] * 4 + [z2] * 4
    pos, num = [], []
    for i in range(reps):
        for j in range(reps):
            for k in range(reps):
                for b, z in zip(basis, species):
                    pos.append((np.array([i, j, k]) + b) * a)
                    num.append(z)
    pos = np.array(pos) + rng.normal(0.0, jitter_angstrom * ANGSTROM_TO_BOHR, (len(pos), 3))
    cell = np.eye(3) * a * reps
    return {"numbers": np.array(num), "positions": pos, "cell": cell}


def _cell_from_params(a, b, c, alpha, beta, gamma):
    ca, cb, cg = math.cos(alpha), math.cos(beta), math.cos(gamma)
    sg = math.sin(gamma)
    v1 = np.array([a, 0.0, 0.0])
    v2 = np.array([b * cg, b * sg, 0.0])
    cx = c * cb
    cy = c * (ca - cb * cg) / sg
    cz2 = c * c - cx * cx - cy * cy
    if cz2 <= 1e-6 * c * c:
        return None
    return np.array([v1, v2, [cx, cy, math.sqrt(cz2)]])


def random_structure(rng: np.random.Generator, n_atoms: int, zmax: int = 65,
                     min_dist_angstrom: float = 1.8, max_tries: int = 200) -> dict:
    """Triclinic cell, edges U(4,15) A, angles U(60,120) deg, uniform atoms with rejection.

    A cell is redrawn until all ``n_atoms`` fit at the minimum (periodic)
    distance; placement tries each atom up to ``max_tries`` times.
    """
    dmin = min_dist_angstrom * ANGSTROM_TO_BOHR
    while True:
        edges = rng.uniform(4.0, 15.0, 3) * ANGSTROM_TO_BOHR
        ang = np.radians(rng.uniform(60.0, 120.0, 3))
        cell = _cell_from_params(*edges, *ang)
        if cell is None:
            continue
        frac = np.empty((n_atoms, 3))
        placed_n = 0
        ok = True
        shifts = np.array([[i, j, k] for i in (-1, 0, 1) for j in (-1, 0, 1) for k in (-1, 0, 1)], float)
        for _ in range(n_atoms):
            placed = False
            for _t in range(max_tries):
                f = rng.uniform(0.0, 1.0, 3)
                if placed_n:
                    d = (frac[:placed_n, None, :] - f[None, None, :] + shifts[None]) @ cell
                    if np.sqrt((d * d).sum(-1)).min() < dmin:
                        continue
                frac[placed_n] = f
                placed_n += 1
                placed = True
                break
            if not placed:
                ok = False
                break
        if ok:
            break
    numbers = rng.integers(1, zmax + 1, n_atoms)
    pos = frac @ cell
    return {"numbers": numbers, "positions": pos, "cell": cell}


def gamma_centred_grid(cell: np.ndarray, n_atoms: int, kdens: float = 1000.0) -> Tuple[int, int, int]:
    """Per-axis counts ``n_i`` proportional to the reciprocal lengths with ``prod(n) ~ kdens / n_atoms``."""
    target = max(1.0, kdens / n_atoms)
    rec = np.linalg.inv(cell).T
    blen = np.linalg.norm(rec, axis=1)
    scale = (target / np.prod(blen)) ** (1.0 / 3.0)
    n = np.maximum(1, np.rint(blen * scale)).astype(int)
    return int(n[0]), int(n[1]), int(n[2])


def gamma_centred_kpoints(mesh: Tuple[int, int, int]) -> np.ndarray:
    """Fractional k-points ``i/n`` per axis (Gamma included), x slowest."""
    n1, n2, n3 = mesh
    k = np.array([[i / n1, j / n2, l / n3] for i in range(n1) for j in range(n2) for l in range(n3)])
    return k


def uneven_batch(n_structures: int = 256, nmin: int = 2, nmax: int = 64, zmax: int = 65,
                 seed: int = 0, kdens: float = 1000.0) -> List[dict]:
    """Random periodic structures with log-uniform atom counts and Gamma-centred grids."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_structures):
        n = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        st = random_structure(rng, n, zmax=zmax)
        st["mesh"] = gamma_centred_grid(st["cell"], n, kdens)
        st["kpoints"] = gamma_centred_kpoints(st["mesh"])
        out.append(st)
    return out


# ------------------------------------------------------------ serving stream

SERVING_CHUNK = 625        # structures per seeded chunk of the serving request set
SERVING_SEED = 1000        # chunk i is drawn from seed SERVING_SEED + i
SERVING_SHUFFLE_SEED = 5   # one permutation interleaves the chunks


def _serving_chunk(args) -> List[dict]:
    n, seed = args
    return uneven_batch(n, nmin=1, nmax=200, zmax=65, seed=seed)


def serving_requests(n_requests: int, processes: int = 1, chunk: int = SERVING_CHUNK, seed: int = SERVING_SEED,
                     shuffle_seed: int = SERVING_SHUFFLE_SEED) -> List[dict]:
    """Serving request set: structures of 1-200 atoms (log-uniform), Z 1-65, random triclinic
    cells, Gamma-centred grids of ~1000 k-atoms, uniform k-point weights.

    The set is drawn in chunks of ``chunk`` structures, chunk i from ``uneven_batch`` with seed
    ``seed + i``, then shuffled by one seeded permutation.  The result depends only on the
    arguments, not on ``processes`` (worker processes for the chunks, started with ``spawn`` so
    that they are safe after CUDA is initialised)."""
    jobs = [(min(chunk, n_requests - a), seed + i) for i, a in enumerate(range(0, n_requests, chunk))]
    if processes > 1 and len(jobs) > 1:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(min(processes, len(jobs))) as pool:
            parts = pool.map(_serving_chunk, jobs)
    else:
        parts = [_serving_chunk(j) for j in jobs]
    sts = [s for p in parts for s in p]
    sts = [sts[i] for i in np.random.default_rng(shuffle_seed).permutation(len(sts))]
    for st in sts:
        st["weights"] = np.full(len(st["kpoints"]), 1.0 / len(st["kpoints"]))
    return sts


def save_structures(path: str, structures: List[dict]) -> None:
    """Write structures (numbers, positions, cell, kpoints) to one compressed .npz."""
    np.savez_compressed(path, natoms=np.array([len(s["numbers"]) for s in structures]),
                        nk=np.array([len(s["kpoints"]) for s in structures]),
                        numbers=np.concatenate([np.asarray(s["numbers"]) for s in structures]),
                        positions=np.concatenate([np.asarray(s["positions"]) for s in structures]),
                        cells=np.stack([np.asarray(s["cell"]) for s in structures]),
                        kpoints=np.concatenate([np.asarray(s["kpoints"]) for s in structures]))


def load_structures(path: str) -> List[dict]:
    """Read a file written by ``save_structures``; k-point weights are uniform."""
    with np.load(path) as z:
        arr = {k: z[k] for k in z.files}      # each z[k] decompresses the whole array: read once
    out, a, k = [], 0, 0
    for i, (na, nk) in enumerate(zip(arr["natoms"].tolist(), arr["nk"].tolist())):
        out.append({"numbers": arr["numbers"][a:a + na].copy(), "positions": arr["positions"][a:a + na].copy(),
                    "cell": arr["cells"][i].copy(), "kpoints": arr["kpoints"][k:k + nk].copy(),
                    "weights": np.full(nk, 1.0 / nk)})
        a += na
        k += nk
    return out
