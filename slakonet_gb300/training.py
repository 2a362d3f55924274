"""Parameter fitting on the GB300 path: one batched forward, the hand-written adjoint backward.

``train_step`` mirrors one epoch step of the reference's
``train_multi_vasp_skf_parameters`` (slakonet/optim.py:1570-1855):
``apply_constraints``, per-structure losses weighted by atom count,
``1e-10 * sum(theta^2)`` regularisation, backward, gradient clipping at 2.0,
AdamW and ReduceLROnPlateau.  The reference evaluates one structure at a
time and differentiates with autograd; here the whole batch runs in one
launch sequence and the gradient comes from ``adjoint.py``.  The reference
computes a DOS MSE, a DOS MAE and a peak term for each dataset, then keeps
only the band-gap absolute error as the dataset loss
(slakonet/optim.py:1700-1718); ``dos_weight=0`` gives exactly that loss.  The
default, Gaussian-DOS MSE plus band-gap absolute error, is the loss of the
64-structure fitting workload.
"""
from __future__ import annotations

import time
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from . import adjoint as A
from . import synthetic as syn
from .model import MultiElementSkfParameterOptimizer

DOS_RANGE = (-20.0, 10.0)
DOS_POINTS = 1000


def fitting_batch(n_structures: int = 64, nmin: int = 4, nmax: int = 32, zmax: int = 30, seed: int = 0,
                  kdens: float = 1000.0) -> List[dict]:
    """Random periodic structures (as the uneven batch), 4-32 atoms, Z <= 30."""
    sts = syn.uneven_batch(n_structures, nmin=nmin, nmax=nmax, zmax=zmax, seed=seed, kdens=kdens)
    for st in sts:
        st["weights"] = np.full(len(st["kpoints"]), 1.0 / len(st["kpoints"]))
    return sts


def perturbed_targets(tables: dict, structures: Sequence[dict], shell_dict, device, rel: float = 0.05,
                      seed: int = 1):
    """Target DOS [S, 1000] and gaps [S] from the same path with amplitudes scaled by 1 + N(0, rel)."""
    target_model = MultiElementSkfParameterOptimizer.from_tables(syn.perturb_tables(tables, rel, seed))
    res = target_model.compute_properties_batch(structures, shell_dict, device, dos_range=DOS_RANGE,
                                                dos_points=DOS_POINTS, dos_window=9.0)
    from .engine import STAT
    return res.dos.clone(), res.stats[:, STAT["gap_ev"]].clone()


def train_step(model: MultiElementSkfParameterOptimizer, optimizer: torch.optim.Optimizer,
               structures: Sequence[dict], dos_target: torch.Tensor, gap_target: torch.Tensor, shell_dict,
               device, scheduler=None, weight_by_natoms: bool = True, dos_weight: float = 1.0,
               gap_weight: float = 1.0, clip: float = 2.0) -> Dict[str, float]:
    t0 = time.perf_counter()
    optimizer.zero_grad()
    model.apply_constraints()
    eig, dos, gap, res = A.differentiable_properties(model, structures, shell_dict, device, dos_range=DOS_RANGE,
                                                     dos_points=DOS_POINTS, dos_window=9.0)
    per = dos_weight * ((dos - dos_target) ** 2).mean(1) + gap_weight * (gap - gap_target).abs()
    w = torch.as_tensor(np.diff(res.plan.atom_ptr).astype(np.float64) if weight_by_natoms
                        else np.ones(res.plan.n_struct), device=per.device)
    # a structure whose Fermi search diverged (NaN, as in the reference) or whose S(k) is not
    # positive definite drops out of the batch; the reference skips the whole step instead
    ok = torch.isfinite(per) & torch.isfinite(dos_target).all(1) & torch.isfinite(gap_target)
    per = torch.where(ok, per, torch.zeros_like(per))
    w = torch.where(ok, w, torch.zeros_like(w))
    batch_loss = (per * w).sum() / w.sum().clamp(min=1e-300)
    params = [p for p in model.parameters()]
    # 1e-10 * sum(theta^2): value from fused norms, gradient 2e-10 * theta added after backward
    with torch.no_grad():
        reg = float(torch.stack(torch._foreach_norm(params)).pow(2).sum())
    t1 = time.perf_counter()
    batch_loss.backward()
    with torch.no_grad():
        grads = [p.grad if p.grad is not None else torch.zeros_like(p) for p in params]
        for p, gr in zip(params, grads):
            if p.grad is None:
                p.grad = gr
        torch._foreach_add_(grads, params, alpha=2e-10)
    loss = batch_loss.detach() + 1e-10 * reg
    torch.nn.utils.clip_grad_norm_(params, max_norm=clip)
    optimizer.step()
    if scheduler is not None:
        scheduler.step(loss.detach())
    if torch.cuda.is_available():
        torch.cuda.synchronize()
    t2 = time.perf_counter()
    st = res.state or {}
    return {"loss": float(loss.detach()), "batch_loss": float(batch_loss.detach()), "forward_s": t1 - t0,
            "structures_used": int(ok.sum()),
            "backward_s": t2 - t1, "degenerate_pairs": int(st.get("degenerate_pairs", 0))}


def fit(model: MultiElementSkfParameterOptimizer, structures: Sequence[dict], dos_target: torch.Tensor,
        gap_target: torch.Tensor, shell_dict, device, num_epochs: int = 100, learning_rate: float = 1e-5,
        batch_size: Optional[int] = None, save_directory: Optional[str] = None, early_stopping_patience: int = 20,
        seed: int = 0, log=None) -> Dict[str, object]:
    """The reference's fitting loop (``train_multi_vasp_skf_parameters``, slakonet/optim.py:1570-1855) around
    ``train_step``: AdamW at ``learning_rate``; ReduceLROnPlateau (factor 0.8, patience 10) stepped with each
    epoch's loss; each epoch on all structures, or on ``batch_size`` of them drawn at random (seeded); the
    best model so far kept and, with ``save_directory``, written as ``best_model.pt`` in the reference's
    ultra-compact checkpoint format; a stop after ``early_stopping_patience`` epochs without improvement;
    the final model and the loss history (``final_model.pt``, ``training_history.json``) at the end.  The
    reference reads its targets from VASP runs; here they are passed in (DOS ``[S, 1000]`` and gaps ``[S]``
    in eV, as ``perturbed_targets`` makes).  Returns the history and the best loss."""
    import json
    import os
    optimizer = torch.optim.AdamW(model.parameters(), lr=learning_rate)
    scheduler = torch.optim.lr_scheduler.ReduceLROnPlateau(optimizer, mode="min", factor=0.8, patience=10)
    rng = np.random.default_rng(seed)
    history: List[dict] = []
    best_loss, best_epoch, stale = float("inf"), -1, 0
    best_state = None
    if save_directory:
        os.makedirs(save_directory, exist_ok=True)
    for epoch in range(num_epochs):
        if batch_size is not None and batch_size < len(structures):
            idx = np.sort(rng.choice(len(structures), size=batch_size, replace=False))
        else:
            idx = np.arange(len(structures))
        sel = torch.as_tensor(idx, device=dos_target.device)
        rec = train_step(model, optimizer, [structures[i] for i in idx], dos_target[sel], gap_target[sel],
                         shell_dict, device, scheduler=scheduler)
        loss = rec["loss"]
        history.append({"epoch": epoch, "loss": loss, "lr": optimizer.param_groups[0]["lr"],
                        "structures": int(rec.get("structures_used", len(idx)))})
        if log is not None:
            log(history[-1])
        if loss < best_loss:
            best_loss, best_epoch, stale = loss, epoch, 0
            best_state = {k: v.detach().clone() for k, v in model.state_dict().items()}
            if save_directory:
                model.save_ultra_compact(os.path.join(save_directory, "best_model.pt"))
        else:
            stale += 1
        if stale >= early_stopping_patience:
            break
    if save_directory:
        model.save_ultra_compact(os.path.join(save_directory, "final_model.pt"))
        with open(os.path.join(save_directory, "training_history.json"), "w") as f:
            json.dump({"history": history, "best_loss": best_loss, "best_epoch": best_epoch}, f, indent=1)
    return {"history": history, "best_loss": best_loss, "best_epoch": best_epoch, "best_state": best_state}
