"""The atom-pair Bloch kernel (skn_bloch_pairs) against the problem-major one (skn_bloch) on a GB300.

Both sum the same bonds in the same order, so with lower = 0 the matrices must be bitwise equal, and
with lower = 1 the entries on or below the diagonal must be bitwise equal while the strict upper
triangle keeps what the buffer held before the call.
"""
import numpy as np
import pytest
import torch

from slakonet_gb300 import engine as E, synthetic as syn
from slakonet_gb300._lib import call, ptr

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _inputs():
    sts = syn.uneven_batch(12, nmin=1, nmax=30, zmax=40, seed=21, kdens=200.0)
    zs = sorted({int(z) for s in sts for z in s["numbers"]})
    sd = syn.default_shell_dict()
    ts = E.TableSet.from_synthetic(syn.make_tables(zs, sd, seed=21), {z: sd[z] for z in zs}, DEV)
    plan = E.plan_batch(sts, ts)
    eng = E.Engine(ts)
    db = E.DeviceBatch(plan, torch.device(DEV))
    b = eng.bonds(db)
    stream = torch.cuda.current_stream(DEV).cuda_stream
    phases = torch.empty(2 * max(plan.n_phase, 1), dtype=torch.float64, device=DEV)
    call("skn_image_phases", plan.n_struct, ptr(db.rng), ptr(db.kptr), ptr(db.kp), ptr(db.phb), ptr(phases), stream)
    blk_H = torch.empty(max(b["nblk"], 1), dtype=torch.float64, device=DEV)
    blk_S = torch.empty(max(b["nblk"], 1), dtype=torch.float64, device=DEV)
    status = torch.zeros(1, dtype=torch.int32, device=DEV)
    T = ts
    call("skn_sk_blocks", b["nbond"], ptr(b["bond_i"]), ptr(b["bond_j"]), ptr(b["bond_d"]), ptr(b["bond_u"]),
         ptr(b["bond_blk"]), ptr(db.species), len(T.species), ptr(T.sp_nshell), ptr(T.sp_shell_l), ptr(T.sp_norb),
         ptr(T.tab_index), ptr(T.tab_off), ptr(T.tab_ngrid), ptr(T.tab_step), ptr(T.tab_H), ptr(T.tab_S),
         ptr(blk_H), ptr(blk_S), ptr(status), stream)
    return plan, db, b, phases, blk_H, blk_S, stream


def _old(plan, db, b, phases, blk_H, blk_S, stream):
    H = torch.zeros(2 * plan.hs_total, dtype=torch.float64, device=DEV)
    S = torch.zeros_like(H)
    call("skn_bloch", len(plan.prob_n), ptr(db.ps), ptr(db.pk), ptr(db.hs_off), ptr(db.atom_ptr), ptr(db.orb_ptr),
         ptr(db.orb_atom), ptr(db.aoff), ptr(db.norb), ptr(db.pair_base), ptr(b["pair_ptr"]), ptr(b["bond_img"]),
         ptr(b["bond_blk"]), ptr(blk_H), ptr(blk_S), ptr(db.rng), ptr(db.phb), ptr(phases), ptr(db.onsite),
         plan.max_n, ptr(H), ptr(S), stream)
    return H, S


def _pairs(plan, db, b, phases, blk_H, blk_S, stream, lower, fill):
    H = torch.full((2 * plan.hs_total,), fill, dtype=torch.float64, device=DEV)
    S = torch.full_like(H, fill)
    units, unit_base = (db.bloch_units_lower, db.bloch_unit_base_lower) if lower else (db.bloch_units, db.bloch_unit_base)
    call("skn_bloch_pairs", plan.n_struct, units, ptr(unit_base), ptr(db.kptr), ptr(db.hs_off),
         ptr(db.atom_ptr),
         ptr(db.orb_ptr), ptr(db.aoff), ptr(db.norb), ptr(db.pair_base), ptr(b["pair_ptr"]), ptr(b["bond_img"]),
         ptr(b["bond_blk"]), ptr(blk_H), ptr(blk_S), ptr(db.rng), ptr(db.phb), ptr(phases), ptr(db.onsite),
         lower, ptr(H), ptr(S), stream)
    return H, S


def _lower_mask(plan):
    parts = []
    for n in plan.prob_n:
        i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")   # element (row i, column j)
        parts.append((i >= j).T.reshape(-1))                            # column-major order
    m = np.concatenate(parts)
    return torch.as_tensor(np.repeat(m, 2), device=DEV)                 # real and imaginary parts


def test_pairs_kernel_bitwise_equal_to_problem_kernel():
    args = _inputs()
    plan = args[0]
    H0, S0 = _old(*args)
    H1, S1 = _pairs(*args, lower=0, fill=0.0)
    torch.cuda.synchronize()
    assert torch.equal(H0, H1) and torch.equal(S0, S1)
    H2, S2 = _pairs(*args, lower=1, fill=-3.0)
    torch.cuda.synchronize()
    low = _lower_mask(plan)
    assert torch.equal(H2[low], H0[low]) and torch.equal(S2[low], S0[low])
    assert bool((H2[~low] == -3.0).all()) and bool((S2[~low] == -3.0).all())
    print(f"{len(plan.prob_n)} problems, n up to {plan.max_n}: pair kernel bitwise equal (full and lower)")
