"""Differentiable properties: forward on the CUDA path, hand-written adjoint backward.

``differentiable_properties`` returns eigenvalues, DOS and band gap as
tensors attached to the model's ``h_params`` / ``s_params``; calling
``backward`` on any loss built from them runs the adjoint kernels
(``csrc/adjoint.cu``): DOS backward, band-gap selection, weighted
eigenvector projectors, Bloch-sum adjoint, and the pull-back through the
rotations and splines onto the table entries.  The reference obtains the
same gradients with autograd through its whole forward graph
(slakonet/optim.py:1656-1772, slakonet/utils.py:387-473).

As in the reference, the Fermi level is not differentiated (fermi_search
detaches it, slakonet/fermi.py:191-196), the band gap's gradient flows to
the two band-edge eigenvalues that define it, and a metal's gap (zero) has
no gradient.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import numpy as np
import torch

from . import _lib
from ._lib import call, ptr
from . import engine as E

H2E = 27.211


class _Properties(torch.autograd.Function):
    @staticmethod
    def forward(ctx, holder, *params):
        eng, db, dos_kw = holder["engine"], holder["db"], holder["dos_kw"]
        res = eng.execute(db, vectors=True, keep_state=True, **dos_kw)
        eng.check_tables()
        holder["res"] = res
        ctx.holder = holder
        gap = res.stats[:, E.STAT["gap_ev"]].clone()
        return res.eig, res.dos, gap

    @staticmethod
    def backward(ctx, g_eig, g_dos, g_gap):
        holder = ctx.holder
        res, eng = holder["res"], holder["engine"]
        grads = adjoint(eng, res, g_eig, g_dos, g_gap)
        return (None, *grads)


def adjoint(eng: "E.Engine", res: "E.BatchResult", g_eig=None, g_dos=None, g_gap=None):
    """Parameter gradients (in ``eng.tables.param_slices`` order) for upstream gradients
    of the flat eigenvalues, the DOS ``[S, npts]`` and the gap ``[S]`` (eV)."""
    T = eng.tables
    plan = res.plan
    st = res.state
    db = st["db"]
    dev = eng.device
    stream = torch.cuda.current_stream(dev).cuda_stream
    S = plan.n_struct
    g = torch.zeros(max(plan.eig_total, 1), dtype=torch.float64, device=dev)
    if g_eig is not None:
        g += g_eig.to(torch.float64)
    if g_dos is not None:
        lo, hi, npts, sigma, window = st["dos_args"]
        gd = g_dos.to(torch.float64).contiguous()
        max_count = int((plan.nk.astype(np.int64) * plan.nb).max())
        call("skn_dos_backward", S, ptr(db.eos), ptr(db.nk), ptr(db.nb), ptr(db.kwoff), ptr(db.kw), ptr(res.eig),
             ptr(res.mu), lo, hi, npts, sigma, window, ptr(gd), ptr(g), max_count, stream)
    if g_gap is not None:
        stats = res.stats
        vf = stats[:, E.STAT["vbm_flat"]]
        cf = stats[:, E.STAT["cbm_flat"]]
        ok = (vf >= 0) & (cf >= 0)
        base = db.eos
        gg = g_gap.to(torch.float64) * H2E
        iv = (base + vf.clamp(min=0).long())[ok]
        ic = (base + cf.clamp(min=0).long())[ok]
        g.index_add_(0, iv, -gg[ok])
        g.index_add_(0, ic, gg[ok])
    st["degenerate_pairs"] = _degenerate_pairs(plan, res.eig, g)
    n_prob = len(plan.prob_n)
    Gm = torch.empty(2 * max(plan.hs_total, 1), dtype=torch.float64, device=dev)
    Fm = torch.empty_like(Gm)
    vec = torch.view_as_real(res.vec).reshape(-1)
    g = torch.nan_to_num(g, nan=0.0, posinf=0.0, neginf=0.0)
    call("skn_adj_projectors", n_prob, ptr(db.n), ptr(db.hs_off), ptr(db.eoff), ptr(vec), ptr(res.eig), ptr(g),
         ptr(res.eig_status), ptr(Gm), ptr(Fm), stream)
    nbond = st["nbond"]
    dtab_H = torch.zeros_like(T.tab_H)
    dtab_S = torch.zeros_like(T.tab_S)
    if nbond:
        gbH = torch.empty(max(st["nblk"], 1), dtype=torch.float64, device=dev)
        gbS = torch.empty_like(gbH)
        atom_struct = getattr(db, "atom_struct", None)
        if atom_struct is None:
            db.atom_struct = E._i32(np.repeat(np.arange(S, dtype=np.int32), np.diff(plan.atom_ptr)), dev)
            db.struct_prob0 = E._i32(np.concatenate([[0], np.cumsum(plan.nk)[:-1]]), dev)
        call("skn_adj_bloch", nbond, ptr(st["bond_i"]), ptr(st["bond_j"]), ptr(st["bond_img"]), ptr(st["bond_blk"]),
             ptr(db.atom_struct), ptr(db.aoff), ptr(db.norb), ptr(db.struct_prob0), ptr(db.nk), ptr(db.nb),
             ptr(db.hs_off), ptr(db.rng), ptr(db.phb), ptr(st["phases"]), ptr(Gm), ptr(Fm), ptr(gbH), ptr(gbS),
             stream)
        call("skn_adj_tables", nbond, ptr(st["bond_i"]), ptr(st["bond_j"]), ptr(st["bond_d"]), ptr(st["bond_u"]),
             ptr(st["bond_blk"]), ptr(db.species), len(T.species), ptr(T.sp_nshell), ptr(T.sp_shell_l),
             ptr(T.sp_norb), ptr(T.tab_index), ptr(T.tab_off), ptr(T.tab_ngrid), ptr(T.tab_step), ptr(gbH), ptr(gbS),
             ptr(dtab_H), ptr(dtab_S), stream)
    grads = []
    for tensor, kind, off, numel in T.param_slices:
        src = dtab_H if kind == "H" else dtab_S
        grads.append(src[off: off + numel].view(tensor.shape).to(tensor.device))
    return grads


def _degenerate_pairs(plan, eig, g, tol: float = 1e-8) -> int:
    """Adjacent bands at one k closer than ``tol`` Hartree whose loss weights differ.

    For such a pair the derivative of each eigenvalue separately is not
    defined; the projector form used here returns the derivative of the
    weighted sum over the degenerate subspace, which is exact only when the
    weights agree.  The count is reported so callers can tell.
    """
    if plan.eig_total < 2:
        return 0
    nb = np.repeat(plan.nb, plan.nk.astype(np.int64) * plan.nb)
    pos = np.concatenate([np.arange(int(k) * int(b)) % int(b) for k, b in zip(plan.nk, plan.nb)])
    valid = torch.as_tensor((pos[:-1] < nb[:-1] - 1), device=eig.device)
    de = (eig[1:plan.eig_total] - eig[:plan.eig_total - 1]).abs()
    dg = (g[1:plan.eig_total] - g[:plan.eig_total - 1]).abs()
    gscale = float(g.abs().max()) if plan.eig_total else 0.0
    flag = valid & (de < tol) & (dg > 1e-9 * max(gscale, 1e-300))
    return int(flag.sum())


def differentiable_properties(model, structures: Sequence[dict], shell_dict=None, device="cuda",
                              dos_range=(-20.0, 10.0), dos_points: int = 1000, dos_sigma: float = 0.1,
                              dos_window: float = 9.0, cutoff: float = E.CUTOFF_BOHR):
    """(eigenvalues_flat, dos [S, npts], gap [S] eV, BatchResult) with gradients to the model's tables."""
    from .model import _default_shell_dict
    device = torch.device(device)
    shell_dict = shell_dict if shell_dict is not None else _default_shell_dict()
    zs = sorted({int(z) for st in structures for z in np.asarray(st["numbers"]).reshape(-1)})
    ts = model.table_set(shell_dict, device, zs)
    eng = E.Engine(ts, cutoff)
    plan = E.plan_batch(structures, ts, cutoff)
    db = E.DeviceBatch(plan, device)
    holder = {"engine": eng, "db": db,
              "dos_kw": dict(dos_range=dos_range, dos_points=dos_points, dos_sigma=dos_sigma, dos_window=dos_window)}
    params = [t for t, _, _, _ in ts.param_slices]
    eig, dos, gap = _Properties.apply(holder, *params)
    return eig, dos, gap, holder["res"]
