"""CPU oracle for the SlakoNet electronic-structure path (test infrastructure).

THIS MODULE IS TEST INFRASTRUCTURE.  It is a numpy restatement of the
reference's algorithm and is imported only by ``tests/``, by
``__graft_entry__.smoke()`` and by ``bench.py`` (its CPU-baseline leg and the
``--impl reference`` arm), always as the parity reference or the timed CPU baseline,
never as part of the product path.  The product path (``slakonet_gb300``)
runs the CUDA kernels and fails loudly without them.

Parity pin: the functions here are checked against golden vectors produced
by running the reference itself (``tests/golden/make_golden.py``) in
``tests/test_oracle_golden.py``.

Each function cites the reference file:line it restates (paths relative to
the reference project).  Units: Bohr, Hartree; eV only where the reference
converts with H2E = 27.211 (slakonet/main.py:34).
"""
from __future__ import annotations

import math
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

H2E = 27.211  # slakonet/main.py:34


# --------------------------------------------------------------- k-points

def mp_kpoints(mesh: Sequence[int]) -> Tuple[np.ndarray, np.ndarray]:
    """Offset Monkhorst-Pack grid ``0.5/n + i/n`` per axis, x slowest.

    Restates ``Periodic._super_sampling`` (slakonet/atoms.py:394-446).
    Returns fractional k-points ``[nk, 3]`` and weights ``1/nk``.
    """
    n1, n2, n3 = (int(v) for v in mesh)
    ks = []
    for i in range(n1):
        for j in range(n2):
            for l in range(n3):
                ks.append([0.5 / n1 + i * (1.0 / n1), 0.5 / n2 + j * (1.0 / n2), 0.5 / n3 + l * (1.0 / n3)])
    k = np.array(ks, dtype=np.float64)
    return k, np.full(len(k), 1.0 / len(k))


def klines_kpoints(klines: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
    """Points along band-structure segments ``[k1(3), k2(3), N]``.

    Restates ``Periodic._klines`` (slakonet/atoms.py:448-502): ``N`` points
    ``k1 + i (k2 - k1)/(N - 1)`` per segment, weights ``1/total``.  A
    segment with ``N == 1`` divides by zero exactly as the reference does.
    """
    kl = np.asarray(klines, dtype=np.float64).reshape(-1, 7)
    pts = []
    for row in kl:
        n = int(row[6])
        d = row[3:6] - row[0:3]
        if n >= 1:
            with np.errstate(divide="ignore", invalid="ignore"):
                d = d / (row[6] - 1.0)
        for i in range(n):
            pts.append(row[0:3] + d * i)
    k = np.array(pts, dtype=np.float64).reshape(-1, 3)
    return k, np.full(len(k), 1.0 / max(len(k), 1))


# ------------------------------------------------------------ image list

def cell_translations(cell: np.ndarray, rcut_images: float) -> np.ndarray:
    """Integer cell translations ``-(e + floor(rc |a*_i|)) .. +(...)``.

    Restates ``Periodic.get_cell_translations`` (slakonet/atoms.py:165-215)
    with the extension of one cell on each side; x slowest.
    """
    inv = np.linalg.inv(cell).T  # rows: reciprocal vectors / 2pi   (atoms.py:336-357)
    r = np.floor(rcut_images * np.linalg.norm(inv, axis=1)) + 1.0
    rng = [np.arange(-int(v), int(v) + 1) for v in r]
    return np.array([[a, b, c] for a in rng[0] for b in rng[1] for c in rng[2]], dtype=np.float64)


def bond_list(positions: np.ndarray, cell: np.ndarray, cutoff: float = 10.0,
              rcut_images: float = 21.0):
    """All directed bonds ``(i, j, T)`` with ``0 < |r_j + T - r_i| < cutoff``.

    Restates the periodic distance tables (slakonet/atoms.py:217-243) and
    the distance mask of ``hs_matrix`` (slakonet/slaterkoster.py:269-276).
    Returns ``i, j, T[int,3], d, u`` where ``u`` is the unit vector from
    atom ``i`` to the image of ``j`` (slakonet/slaterkoster.py:201).
    """
    T = cell_translations(cell, rcut_images)
    rT = T @ cell
    n = len(positions)
    vec = positions[None, None, :, :] + rT[:, None, None, :] - positions[None, :, None, :]  # [c,i,j,3]
    d = np.sqrt((vec * vec).sum(-1))
    mask = (d < cutoff) & (d > 0.0)
    c, i, j = np.nonzero(mask)
    dd = d[c, i, j]
    u = vec[c, i, j] / dd[:, None]
    return i, j, T[c].astype(np.int64), dd, u


# -------------------------------------------------------- interpolation

def _neville_first_point(xa: np.ndarray, ya: np.ndarray, r: np.ndarray) -> np.ndarray:
    """Neville recursion started at the first window point.

    Restates ``poly_interp`` (slakonet/interpolation.py:255-311): the
    nearest-point search there never advances, so the recursion always
    starts from ``ya[0]`` and adds ``c[0]`` at every order.
    ``xa [B, n]``, ``ya [B, n, m]``, ``r [B]``.
    """
    n = xa.shape[1]
    c = ya.copy()
    dd = ya.copy()
    y = ya[:, 0].copy()
    for mm in range(n - 1):
        for ii in range(n - mm - 1):
            r0 = xa[:, ii] - xa[:, ii + mm + 1]
            r1 = (c[:, ii + 1] - dd[:, ii]) / r0[:, None]
            c[:, ii] = (xa[:, ii] - r)[:, None] * r1
            dd[:, ii] = (xa[:, ii + mm + 1] - r)[:, None] * r1
        y = y + c[:, 0]
    return y


def _poly5_zero(y0, y0p, y0pp, xx, dx):
    """5th-order tail to zero (slakonet/interpolation.py:241-252)."""
    dx1 = y0p * dx
    dx2 = y0pp * dx * dx
    dd = 10.0 * y0 - 4.0 * dx1 + 0.5 * dx2
    ee = -15.0 * y0 + 7.0 * dx1 - 1.0 * dx2
    ff = 6.0 * y0 - 3.0 * dx1 + 0.5 * dx2
    xr = xx / dx
    return ((ff * xr + ee) * xr + dd) * xr * xr * xr


def interpolate(table: np.ndarray, step: float, r: np.ndarray, tail: float = 1.0,
                delta_r: float = 1e-5, n_interp: int = 8, n_interp_r: int = 4) -> np.ndarray:
    """Integrals ``[len(r), m]`` from a table ``[m, n_grid]`` on grid ``step*(1..n)``.

    Restates ``PolyInterpU.__call__`` (slakonet/interpolation.py:107-238):
    8-point Neville on the window ending ``n_interp_r`` points past
    ``floor(r/h)`` (clamped to the table), the 5th-order tail for
    ``n_grid <= floor(r/h) <= n_grid - 1 + tail/h``, zero beyond.
    """
    yy = np.asarray(table, dtype=np.float64).T  # [n_grid, m]
    ng, m = yy.shape
    r = np.asarray(r, dtype=np.float64)
    out = np.zeros((len(r), m))
    ind = np.floor(r / step).astype(np.int64)
    pm = ind <= ng
    if pm.any():
        last = ind[pm] + n_interp_r + 1
        last = np.where(last > ng, ng, last)
        last = np.where(last < n_interp + 1, n_interp + 1, last)
        xa = (last[:, None] - n_interp + np.arange(n_interp)[None, :]) * step
        rows = last[:, None] - n_interp - 1 + np.arange(n_interp)[None, :]
        out[pm] = _neville_first_point(xa, yy[rows], r[pm])
    max_ind = ng - 1 + int(tail / step)
    tm = (ind >= ng) & (ind <= max_ind)
    if tm.any():
        r_max = (ng - 1) * step + tail
        dr = r[tm] - r_max
        xa = ((ng - n_interp + np.arange(n_interp)) * step)[None, :]
        yb = yy[ng - n_interp - 1: ng - 1][None]
        x_end = xa[:, n_interp - 1]
        y0 = _neville_first_point(xa, yb, x_end - delta_r)[0]
        y2 = _neville_first_point(xa, yb, x_end + delta_r)[0]
        y1 = yy[ng - 2]
        y1p = (y2 - y0) / (2.0 * delta_r)
        y1pp = (y2 + y0 - 2.0 * y1) / (delta_r * delta_r)
        out[tm] = _poly5_zero(y1[None], y1p[None], y1pp[None], dr[:, None], -1.0 * tail)
    return out


# ------------------------------------------------ rotations (real harmonics)

_GL_T, _GL_W = np.polynomial.legendre.leggauss(6)
_NPHI = 12
_PHI = 2.0 * np.pi * np.arange(_NPHI) / _NPHI
_QT = np.repeat(_GL_T, _NPHI)
_QP = np.tile(_PHI, len(_GL_T))
_QST = np.sqrt(1.0 - _QT * _QT)
_QPTS = np.stack([_QST * np.cos(_QP), _QST * np.sin(_QP), _QT], -1)   # [Q,3]
_QW = np.repeat(_GL_W, _NPHI) * (2.0 * np.pi / _NPHI)


def real_harmonics(v: np.ndarray, l: int) -> np.ndarray:
    """Orthonormal real spherical harmonics ``[..., 2l+1]`` at unit vectors ``v``.

    Ordered m = -l..l, i.e. p (y, z, x) and d (xy, yz, z2, xz, x2-y2), the
    orbital order fixed by the reference's rotation tables
    (slakonet/slaterkoster.py:1178-1606).
    """
    x, y, z = v[..., 0], v[..., 1], v[..., 2]
    pi = math.pi
    if l == 0:
        return np.full(v.shape[:-1] + (1,), 0.5 / math.sqrt(pi))
    if l == 1:
        c = math.sqrt(3.0 / (4.0 * pi))
        return np.stack([c * y, c * z, c * x], -1)
    if l == 2:
        c1 = 0.5 * math.sqrt(15.0 / pi)
        c0 = 0.25 * math.sqrt(5.0 / pi)
        c2 = 0.25 * math.sqrt(15.0 / pi)
        return np.stack([c1 * x * y, c1 * y * z, c0 * (3 * z * z - 1), c1 * x * z, c2 * (x * x - y * y)], -1)
    if l == 3:
        a = 0.25 * math.sqrt(35.0 / (2 * pi))
        b = 0.5 * math.sqrt(105.0 / pi)
        c = 0.25 * math.sqrt(21.0 / (2 * pi))
        d = 0.25 * math.sqrt(7.0 / pi)
        e = 0.25 * math.sqrt(105.0 / pi)
        return np.stack([a * y * (3 * x * x - y * y), b * x * y * z, c * y * (5 * z * z - 1),
                         d * z * (5 * z * z - 3), c * x * (5 * z * z - 1), e * z * (x * x - y * y),
                         a * x * (x * x - 3 * y * y)], -1)
    raise ValueError(l)


def frame_for(u: np.ndarray) -> np.ndarray:
    """Rotations ``R [B,3,3]`` with third column ``u`` (bond frame -> system frame)."""
    u = np.asarray(u, dtype=np.float64)
    a = np.zeros_like(u)
    pick = np.argmin(np.abs(u), axis=1)
    a[np.arange(len(u)), pick] = 1.0
    e1 = np.cross(a, u)
    e1 /= np.linalg.norm(e1, axis=1, keepdims=True)
    e2 = np.cross(u, e1)
    return np.stack([e1, e2, u], -1)


def wigner_real(R: np.ndarray, l: int) -> np.ndarray:
    """``D[B, a, m] = <Y_a | Y_m o R^T>`` by exact sphere quadrature.

    This is the rotation of the real harmonics that the reference's
    ``_rot_yz_*`` / ``_rot_xy_*`` tables evaluate in closed form
    (slakonet/slaterkoster.py:1130-1606); here it is obtained by projection
    on a product Gauss-Legendre x trapezoid grid exact to degree 11.
    """
    ya = real_harmonics(_QPTS, l)                    # [Q, a]
    rq = np.einsum("bca,qc->bqa", R, _QPTS)          # R^T r_q  -> [B, Q, 3]
    ym = real_harmonics(rq, l)                        # [B, Q, m]
    return np.einsum("q,qa,bqm->bam", _QW, ya, ym)


def sk_block(u: np.ndarray, la: int, lb: int, ints: np.ndarray, Dcache=None) -> np.ndarray:
    """Rotated SK block ``[B, 2la+1, 2lb+1]`` for ``la <= lb``.

    ``block = D^la diag_m(V_|m|) (D^lb)^T`` restricted to ``|m| <= la``,
    the quantity ``sub_block_rot`` forms from ``sub_block_ref``
    (slakonet/slaterkoster.py:1013-1122).  ``ints [B, la+1]`` ordered
    sigma, pi, delta, phi.
    """
    R = frame_for(u)
    Da = Dcache[la] if Dcache is not None else wigner_real(R, la)
    Db = Dcache[lb] if Dcache is not None else wigner_real(R, lb)
    out = np.zeros((len(u), 2 * la + 1, 2 * lb + 1))
    for m in range(-la, la + 1):
        v = ints[:, abs(m)]
        out += v[:, None, None] * Da[:, :, m + la][:, :, None] * Db[:, :, m + lb][:, None, :]
    return out


# ------------------------------------------------------------- H(k), S(k)

def orbital_layout(numbers: Sequence[int], shell_dict: Dict[int, List[int]]):
    """Orbital offsets per atom and per shell (slakonet/basis.py:115-153)."""
    atom_off, shells = [], []
    o = 0
    for a, z in enumerate(numbers):
        atom_off.append(o)
        for l in shell_dict[int(z)]:
            shells.append((a, l, o))
            o += 2 * l + 1
    return np.array(atom_off), shells, o


def real_space_blocks(structure: dict, tables: dict, shell_dict: Dict[int, List[int]],
                      cutoff: float = 10.0, kind: str = "H"):
    """Bond list plus the dense real-space contribution of every bond.

    For the shell pair ``(a on i, b on j)`` of bond ``(i, j, T)`` with
    direction ``u``: if ``la < lb``, or ``la == lb`` and ``i <= j``, the block
    is ``B[(Zi,Zj),(la,lb)](u)``; otherwise it is
    ``(-1)^(la+lb) B[(Zj,Zi),(lb,la)](u)^T``.  This is the real-space form of
    the reference's upper-triangle assembly plus conjugate fill
    (slakonet/slaterkoster.py:204-405): the lower blocks it fills with
    ``conj`` come from the reversed bond and the reversed table.
    Returns ``(i, j, T, blocks)`` with ``blocks [nb, n_i_orb, n_j_orb]``.
    """
    numbers = [int(z) for z in structure["numbers"]]
    i, j, T, d, u = bond_list(structure["positions"], structure["cell"], cutoff)
    step = tables["step"]
    norb = [sum(2 * l + 1 for l in shell_dict[z]) for z in numbers]
    R = frame_for(u) if len(u) else np.zeros((0, 3, 3))
    D = {l: (wigner_real(R, l) if len(u) else None) for l in range(4)}
    out = []
    # group bonds by (Zi, Zj) for vectorised interpolation
    zi = np.array([numbers[a] for a in i], dtype=np.int64)
    zj = np.array([numbers[a] for a in j], dtype=np.int64)
    blocks = [np.zeros((norb[a], norb[b])) for a, b in zip(i, j)]
    for (A, B) in sorted(set(zip(zi.tolist(), zj.tolist()))):
        sel = np.nonzero((zi == A) & (zj == B))[0]
        la_list = shell_dict[A]
        lb_list = shell_dict[B]
        oa = np.cumsum([0] + [2 * l + 1 for l in la_list])
        ob = np.cumsum([0] + [2 * l + 1 for l in lb_list])
        for sa, la in enumerate(la_list):
            for sb, lb in enumerate(lb_list):
                lo, hi = min(la, lb), max(la, lb)
                direct_mask = np.ones(len(sel), bool) if la < lb else (
                    np.zeros(len(sel), bool) if la > lb else (i[sel] <= j[sel]))
                for direct in (True, False):
                    s2 = sel[direct_mask] if direct else sel[~direct_mask]
                    if len(s2) == 0:
                        continue
                    if direct:
                        tab = tables["pairs"][(A, B)][kind][(la, lb)]
                    else:
                        tab = tables["pairs"][(B, A)][kind][(lb, la)]
                    ints = interpolate(tab, step, d[s2])
                    Dl = {l: D[l][s2] for l in (la, lb)}
                    blk = np.zeros((len(s2), 2 * la + 1, 2 * lb + 1))
                    for m in range(-lo, lo + 1):
                        v = ints[:, abs(m)]
                        blk += v[:, None, None] * Dl[la][:, :, m + la][:, :, None] * Dl[lb][:, :, m + lb][:, None, :]
                    if not direct:
                        blk = blk * (-1.0) ** (la + lb)
                    for q, b_ in enumerate(s2):
                        blocks[b_][oa[sa]:oa[sa + 1], ob[sb]:ob[sb + 1]] = blk[q]
    return i, j, T, blocks


def onsite_vector(numbers: Sequence[int], tables: dict, shell_dict, kind: str = "H") -> np.ndarray:
    """Diagonal on-site terms (slakonet/skfeed.py:675-739, slaterkoster.py:781-831).

    H: the homonuclear table's per-l on-site energy repeated ``2l+1`` times,
    taken by position ``l`` of ``on_sites``; S: ones.
    """
    out = []
    for z in numbers:
        z = int(z)
        for l in shell_dict[z]:
            if kind == "H":
                out.extend([tables["elements"][z]["on_sites"][l]] * (2 * l + 1))
            else:
                out.extend([1.0] * (2 * l + 1))
    return np.array(out, dtype=np.float64)


def hk_sk(structure: dict, tables: dict, shell_dict, kpoints: np.ndarray, cutoff: float = 10.0, blocks=None):
    """``H(k), S(k)`` as ``[nk, n, n]`` complex128.

    ``M(k) = diag(onsite) + sum_bonds block * exp(i 2 pi k . T)``: the Bloch
    sum of ``_pe_sk_data2`` (slakonet/slaterkoster.py:971-1010) with the
    phase of ``Periodic.phase`` (slakonet/atoms.py:543-558).  ``blocks``, when
    given, is ``(real_space_blocks(.., "H"), real_space_blocks(.., "S"))`` of
    this structure, which do not depend on k (the reference also builds them
    once per structure).
    """
    numbers = [int(z) for z in structure["numbers"]]
    atom_off, _, n = orbital_layout(numbers, shell_dict)
    kpoints = np.asarray(kpoints, dtype=np.float64).reshape(-1, 3)
    res = []
    for q, kind in enumerate(("H", "S")):
        i, j, T, blocks_k = (blocks[q] if blocks is not None
                             else real_space_blocks(structure, tables, shell_dict, cutoff, kind))
        M = np.zeros((len(kpoints), n, n), dtype=np.complex128)
        if len(i):
            ph = np.exp(1j * (2.0 * np.pi * kpoints) @ T.T.astype(np.float64))   # [nk, nb]
            for b, (a1, a2) in enumerate(zip(i, j)):
                blk = blocks_k[b]
                o1, o2 = atom_off[a1], atom_off[a2]
                M[:, o1:o1 + blk.shape[0], o2:o2 + blk.shape[1]] += ph[:, b, None, None] * blk[None]
        idx = np.arange(n)
        M[:, idx, idx] += onsite_vector(numbers, tables, shell_dict, kind)[None, :]
        res.append(M)
    return res[0], res[1]


# ----------------------------------------------------------- eigensolve

def eigh_generalized(H: np.ndarray, S: np.ndarray, vectors: bool = False):
    """Cholesky-reduced generalized Hermitian eigensolve, batched over k.

    Restates ``eighb(..., scheme="chol")`` (slakonet/utils.py:741-783):
    zero rows/columns get a unit diagonal, ``L = chol(S)``,
    ``L^-1 = solve(L, I)``, ``C = L^-1 H L^-H``, ``eigh(C)``, ``v = L^-H v'``.
    Raises ``np.linalg.LinAlgError`` where ``S(k)`` is not positive definite
    (the reference drops that k-point, slakonet/main.py:174-184).
    """
    H = np.array(H, dtype=np.complex128, copy=True)
    S = np.array(S, dtype=np.complex128, copy=True)
    n = H.shape[-1]
    eye = np.eye(n, dtype=np.complex128)
    for M in (H, S):
        z = (M == 0)
        msk = z.all(-1) & z.all(-2)
        if msk.any():
            idx = np.arange(n)
            M[..., idx, idx] += msk.astype(np.float64)
    L = np.linalg.cholesky(S)
    Li = np.linalg.solve(L, np.broadcast_to(eye, L.shape))
    LiH = np.conj(np.swapaxes(Li, -1, -2))
    C = Li @ H @ LiH
    if vectors:
        w, v = np.linalg.eigh(C)
        return w, LiH @ v
    return np.linalg.eigvalsh(C)


# ------------------------------------------------------- Fermi, gap, DOS

def fermi_search(eig: np.ndarray, weights: np.ndarray, n_electrons: float, kT: float = 0.01,
                 tol: float = 1e-6, max_iter: int = 100):
    """Half-step Newton search for the Fermi level.

    Restates ``fermi_search`` (slakonet/fermi.py:139-198) including the
    exact autograd derivative of ``1/(exp((e-mu)/kT)+1)``
    (slakonet/fermi.py:201-215): ``grad = sum 2(N-Ne)*2 w occ^2 exp(x) / kT``.
    Returns ``(mu, iterations, converged)``; ``mu`` may be NaN as in the
    reference when the iteration diverges.
    """
    eig = np.asarray(eig, dtype=np.float64)
    w = np.asarray(weights, dtype=np.float64)[:, None]
    mu = eig.mean()
    with np.errstate(over="ignore", invalid="ignore", divide="ignore"):
        for it in range(max_iter):
            t3 = np.exp((eig - mu) / kT)
            occ = (1.0 / (t3 + 1.0)) * 1.0
            total = 2.0 * (occ * w).sum()
            diff = total - n_electrons
            loss = diff ** 2
            g_sum = 2.0 * (2.0 * diff)
            grad = (((g_sum * w) * 1.0) * (occ * occ) * t3 / kT).sum()
            if abs(grad) < tol:
                return mu, it, True
            mu = mu - loss / (grad + 1e-12)
    return mu, max_iter, False


def band_gap(eig: np.ndarray, mu: float) -> dict:
    """``calculate_band_gap`` (slakonet/main.py:637-707), energies in eV.

    Raises ``ValueError`` where the reference's empty ``max``/``min`` raises
    (no occupied or no empty state, or a NaN Fermi level).
    """
    e = eig * H2E
    f = mu * H2E
    occ = e < f
    unocc = e >= f
    if (np.abs(e - f) < 1e-3).any():
        return {"gap": 0.0, "vbm": f, "cbm": f, "direct": False, "vbm_kpoint": 0, "cbm_kpoint": 0,
                "metal": True}
    if not occ.any() or not unocc.any():
        raise ValueError("empty band selection")
    vbm = e[occ].max()
    cbm = e[unocc].min()
    vk = int(np.argwhere(e == vbm)[0][0])
    ck = int(np.argwhere(e == cbm)[0][0])
    return {"gap": cbm - vbm, "vbm": vbm, "cbm": cbm, "direct": vk == ck, "vbm_kpoint": vk,
            "cbm_kpoint": ck, "metal": False}


def band_structure_props(eig: np.ndarray, mu: float) -> dict:
    """``calculate_band_structure_properties`` (slakonet/main.py:1539-1642)."""
    e = (eig - mu) * H2E
    val = e[e < 0]
    con = e[e >= 0]
    vbm = val.max() if len(val) else -np.inf
    cbm = con.min() if len(con) else np.inf
    vw = (val.max() - val.min()) if len(val) else 0.0
    cw = (con.max() - con.min()) if len(con) else 0.0
    gap = cbm - vbm if (np.isfinite(vbm) and np.isfinite(cbm)) else 0.0
    dg = []
    for ik in range(e.shape[0]):
        b = e[ik]
        kv, kc = b[b < 0], b[b > 0]
        if len(kv) and len(kc):
            dg.append(kc.min() - kv.max())
    mdg = min(dg) if dg else np.inf
    return {"band_gap": gap, "valence_band_width": vw, "conduction_band_width": cw,
            "minimum_direct_gap": (mdg if np.isfinite(mdg) else None),
            "is_direct_semiconductor": (abs(gap - mdg) < 0.01) if np.isfinite(mdg) else False}


def torch_linspace(lo: float, hi: float, n: int) -> np.ndarray:
    """Energy grid of ``torch.linspace`` (slakonet/main.py:740-742).

    torch evaluates ``fma(step, i, lo)`` for the first half and
    ``fma(-step, n-1-i, hi)`` for the rest; the fused multiply-add is
    reproduced exactly with rational arithmetic.
    """
    from fractions import Fraction
    lo, hi = float(lo), float(hi)
    if n == 1:
        return np.array([lo])
    step = (hi - lo) / (n - 1)
    half = n // 2
    fs, flo, fhi = Fraction(step), Fraction(lo), Fraction(hi)
    return np.array([float(fs * i + flo) if i < half else float(fhi - fs * (n - 1 - i)) for i in range(n)])


def gaussian_dos(eig: np.ndarray, weights: np.ndarray, mu: float, energy_range=(-10.0, 10.0),
                 num_points: int = 5000, sigma: float = 0.1) -> Tuple[np.ndarray, np.ndarray]:
    """``calculate_dos`` (slakonet/main.py:709-797): Fermi-shifted eV, Gaussian sigma."""
    grid = torch_linspace(energy_range[0], energy_range[1], num_points)
    e = ((eig - mu) * H2E).reshape(eig.shape[0], -1)
    norm = sigma * math.sqrt(2 * math.pi)
    dos = np.zeros(num_points)
    for ik in range(e.shape[0]):
        x = (grid[None, :] - e[ik][:, None]) / sigma
        dos += weights[ik] * (np.exp(-0.5 * x * x) / norm).sum(0)
    return grid, dos


def atom_projected_dos(eig_ha: np.ndarray, vecs: np.ndarray, atom_types, fermi_ev: float, sigma: float = 0.1,
                       energy_range=(-8.0, 6.0), n_points: int = 1000):
    """Atom-type projected DOS, ``compute_atom_projected_dos`` (slakonet/predict_slakonet.py:119-210).

    eig_ha [nk, nb] Hartree; vecs [nk, n_orb, nb] (component, band), the
    reference's eigenvectors (x^H S x = 1).  The orbitals are split into equal
    contiguous blocks, one per atom (n_orb must divide by the atom count, as in
    the reference, whatever each species' real orbital count); an atom type's
    weight for band b is sum |c_ib|^2 over its blocks.  Each (k, b) adds
    weight * exp(-0.5 ((E - e_kb) / sigma)^2) / (sigma sqrt(2 pi)) on the grid
    E = linspace(energy_range) + E_F (eV); the sum is divided by nk.
    Returns (grid relative to E_F, {type: pdos}, unique types in first-seen order).
    """
    eig = np.asarray(eig_ha) * H2E
    nk, nb = eig.shape
    grid = torch_linspace(energy_range[0], energy_range[1], n_points)
    grid_ev = grid + fermi_ev
    unique = list(dict.fromkeys(atom_types))
    n_orb = vecs.shape[1]
    n_atoms = len(atom_types)
    if n_orb % n_atoms != 0:
        raise ValueError(f"n_orbitals ({n_orb}) not divisible by n_atoms ({n_atoms}).")
    per = n_orb // n_atoms
    idx = {a: [] for a in unique}
    o = 0
    for a in atom_types:
        idx[a].extend(range(o, o + per))
        o += per
    norm = 1.0 / (sigma * np.sqrt(2 * np.pi))
    pdos = {a: np.zeros(n_points) for a in unique}
    w = {a: (np.abs(vecs[:, idx[a], :]) ** 2).sum(1) for a in unique}   # [nk, nb]
    for k in range(nk):
        for b in range(nb):
            g = norm * np.exp(-0.5 * ((grid_ev - eig[k, b]) / sigma) ** 2)
            for a in unique:
                pdos[a] += w[a][k, b] * g
    for a in unique:
        pdos[a] /= nk
    return grid, pdos, unique


def band_energy(eig: np.ndarray, weights: np.ndarray, mu: float, kT_ev: float = 0.025) -> float:
    """Fermi-smeared band energy, ``SimpleDftb._calculate_electronic_energy`` (slakonet/main.py:1430-1448):
    sum_k w_k sum_b f(e_kb) e_kb with f = 1 / (1 + exp((e - mu) / kT)), kT = 0.025 eV, and f = 0
    where e is exactly zero (``fermi_smearing``, slakonet/fermi.py:54-96).  Hartree."""
    kT = kT_ev / H2E
    with np.errstate(over="ignore"):
        occ = 1.0 / (1.0 + np.exp((eig - mu) / kT))
    occ[eig == 0] = 0.0
    return float(np.sum(occ * eig * np.asarray(weights)[:, None]))


def fd_forces(structure: dict, tables: dict, shell_dict, delta: float = 1e-2, mesh=(5, 5, 5)) -> np.ndarray:
    """``_compute_forces_finite_diff`` (slakonet/main.py:198-281): F_ij = -(E(+) - E(-)) / (2 delta), with E
    the plain sum of every eigenvalue (no weights, no occupations) on a ``mesh`` Monkhorst-Pack grid and
    the atom displaced by +-delta Bohr along axis j."""
    k, _ = mp_kpoints(mesh)
    pos = np.asarray(structure["positions"], dtype=np.float64)
    F = np.zeros_like(pos)

    def energy(p):
        st = dict(structure, positions=p)
        H, S = hk_sk(st, tables, shell_dict, k)
        return float(sum(np.sum(eigh_generalized(H[q], S[q])) for q in range(len(k))))

    for i in range(pos.shape[0]):
        for j in range(3):
            pf = pos.copy()
            pf[i, j] += delta
            pb = pos.copy()
            pb[i, j] -= delta
            F[i, j] = -(energy(pf) - energy(pb)) / (2 * delta)
    return F


def properties(eig: np.ndarray, weights: np.ndarray, n_electrons: float,
               dos_range=(-10.0, 10.0), dos_points: int = 5000, dos_sigma: float = 0.1) -> dict:
    """The properties dict of ``get_properties_dict`` (slakonet/main.py:1657-1819)
    plus the ``get_fermi`` extras (slakonet/optim.py:1011-1060), as numpy/float."""
    mu, iters, conv = fermi_search(eig, weights, n_electrons)
    out = {"fermi_converged": conv, "fermi_iterations": iters}
    try:
        bg = band_gap(eig, mu)
        fermi = mu
    except ValueError:
        fermi = 0.0
        bg = {"gap": 0.0, "vbm": 0.0, "cbm": 0.0, "direct": True, "vbm_kpoint": 0, "cbm_kpoint": 0}
    bs = band_structure_props(eig, mu)
    out.update({
        "fermi_energy_eV": fermi * H2E, "fermi_energy_Ha": fermi, "band_gap_eV": bg["gap"],
        "vbm_eV": bg["vbm"], "cbm_eV": bg["cbm"], "is_direct_gap": bg["direct"],
        "vbm_kpoint": bg["vbm_kpoint"], "cbm_kpoint": bg["cbm_kpoint"],
        "valence_band_width_eV": bs["valence_band_width"],
        "conduction_band_width_eV": bs["conduction_band_width"],
        "minimum_direct_gap_eV": bs["minimum_direct_gap"],
        "is_direct_semiconductor": bs["is_direct_semiconductor"],
        "nkpoints": eig.shape[0], "nbands": eig.shape[1], "nelectrons": int(n_electrons),
    })
    grid, dos = gaussian_dos(eig, weights, mu, dos_range, dos_points, dos_sigma)
    fi = int(np.argmin(np.abs(grid)))
    reg = np.abs(grid) < 2.0
    out.update({"dos_energy_grid": grid, "dos_values": dos, "dos_at_fermi": dos[fi],
                "dos_gap_center_eV": grid[reg][int(np.argmin(dos[reg]))],
                "dos_total_states": float(np.trapezoid(dos, grid))})
    occ = eig <= mu
    vb = np.where(occ, eig, -np.inf).max()
    cb = np.where(~occ, eig, np.inf).min()
    out["efermi"] = mu * H2E
    out["bandgap"] = max(cb - vb, 0.0) * H2E
    return out


def n_electrons(numbers: Sequence[int], tables: dict) -> float:
    """Sum of homonuclear-table occupations (slakonet/optim.py:1132-1165)."""
    return float(sum(float(np.sum(tables["elements"][int(z)]["occupations"])) for z in numbers))


def run_structure(structure: dict, tables: dict, shell_dict, kpoints: np.ndarray, weights: np.ndarray,
                  cutoff: float = 10.0, dos_range=(-10.0, 10.0), dos_points: int = 5000,
                  dos_sigma: float = 0.1) -> dict:
    """Whole path for one structure: H(k)/S(k), eigenvalues, properties."""
    H, S = hk_sk(structure, tables, shell_dict, kpoints, cutoff)
    eig = eigh_generalized(H, S)
    ne = n_electrons(structure["numbers"], tables)
    props = properties(eig, weights, ne, dos_range, dos_points, dos_sigma)
    props["eigenvalues"] = eig
    return props
