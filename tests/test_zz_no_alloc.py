"""skn_eigh_gen_vectors_noalloc against skn_eigh_gen_vectors (needs a GB300).

The no-allocation entry point keeps its counters, tridiagonal rows and
inverse-iteration workspace in a fixed library-owned device array.  Two calls
in a row on the same batch must each match the allocating entry point:
eigenvalues within 1e-8 eV, eigenvectors within 1e-10 (same algorithm and
start vectors, so the phase convention is the same), same per-problem status.
Requests above the fixed limits are refused with SKN_ERR_CAPACITY.
"""
import ctypes

import pytest
import torch

from conftest import golden
from _cases import load_case
from slakonet_gb300 import _lib, engine as E, synthetic as syn
from slakonet_gb300._lib import call, ptr

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
EV = 27.211
MAX_N, MAX_ROWS = 512, 262144   # SKN_NOALLOC_MAX_N, SKN_NOALLOC_MAX_ROWS


def _batch(structures, tables, sd):
    ts = E.TableSet.from_synthetic(tables, sd, DEV)
    plan = E.plan_batch(structures, ts)
    eng = E.Engine(ts)
    db = E.DeviceBatch(plan, DEV)
    hs = eng.execute(db, keep_hs=True, hs_only=True)
    return plan, db, hs


def _allocating(plan, db, H0, S0):
    n_prob = len(plan.prob_n)
    H, S = H0.clone(), S0.clone()
    eig = torch.empty(max(plan.eig_total, 1), dtype=torch.float64, device=DEV)
    vec = torch.empty_like(H)
    st = torch.empty(n_prob, dtype=torch.int32, device=DEV)
    tri = torch.empty(4 * max(plan.eig_total, 1), dtype=torch.float64, device=DEV)
    need = ctypes.c_int64(0)
    call("skn_eigh_vectors_scratch_bytes", n_prob, plan.max_n, ctypes.addressof(need))
    scratch = torch.empty(max(need.value // 8, 1), dtype=torch.float64, device=DEV)
    ctr = torch.zeros(2, dtype=torch.int32, device=DEV)
    stream = torch.cuda.current_stream(DEV).cuda_stream
    call("skn_eigh_gen_vectors", n_prob, ptr(db.n), ptr(db.hs_off), ptr(db.eoff), ptr(db.order), ptr(H), ptr(S),
         ptr(eig), ptr(vec), ptr(st), ptr(tri), ptr(scratch), int(need.value), ptr(ctr), plan.max_n, stream)
    torch.cuda.synchronize(DEV)
    return eig, vec, st


def _noalloc(plan, db, H0, S0):
    n_prob = len(plan.prob_n)
    H, S = H0.clone(), S0.clone()
    eig = torch.empty(max(plan.eig_total, 1), dtype=torch.float64, device=DEV)
    vec = torch.empty_like(H)
    st = torch.empty(n_prob, dtype=torch.int32, device=DEV)
    stream = torch.cuda.current_stream(DEV).cuda_stream
    call("skn_eigh_gen_vectors_noalloc", n_prob, ptr(db.n), ptr(db.hs_off), ptr(db.eoff), ptr(db.order), ptr(H),
         ptr(S), ptr(eig), ptr(vec), ptr(st), int(plan.eig_total), plan.max_n, stream)
    torch.cuda.synchronize(DEV)
    return eig, vec, st


def _compare(plan, db, hs):
    eig_a, vec_a, st_a = _allocating(plan, db, hs.H, hs.S)
    assert bool((st_a == 0).all())
    for call_no in (1, 2):
        eig_b, vec_b, st_b = _noalloc(plan, db, hs.H, hs.S)
        de = float((eig_b - eig_a).abs().max()) * EV
        dv = float((vec_b - vec_a).abs().max())
        bitwise = torch.equal(eig_a, eig_b) and torch.equal(vec_a, vec_b)
        print(f"call {call_no}: {len(plan.prob_n)} problems, max n {plan.max_n}: |de| {de:.1e} eV, |dC| {dv:.1e}, "
              f"bitwise {bitwise}")
        assert torch.equal(st_a, st_b)
        assert de <= 1e-8 and dv <= 1e-10


@pytest.mark.parametrize("case", ["si_cfg0", "rand_b"])
def test_noalloc_matches_allocating_entry_on_golden_cases(case):
    g = golden(case)
    st, tables, sd = load_case(g)
    plan, db, hs = _batch([dict(st, kpoints=g["kpoints"])], tables, sd)
    _compare(plan, db, hs)


def test_noalloc_matches_allocating_entry_on_uneven_batch():
    """Problems of up to 270 orbitals: the vector stage runs on 24 CTAs for 416 problems."""
    sts = syn.uneven_batch(12, nmin=2, nmax=60, zmax=30, seed=12, kdens=200.0)
    zs = sorted({int(z) for s in sts for z in s["numbers"]})
    sd = syn.default_shell_dict()
    tables = syn.make_tables(zs, sd, seed=12)
    plan, db, hs = _batch(sts, tables, {z: sd[z] for z in zs})
    assert plan.max_n <= MAX_N and plan.eig_total <= MAX_ROWS
    _compare(plan, db, hs)


def test_noalloc_refuses_sizes_above_its_limits():
    g = golden("rand_c")
    st, tables, sd = load_case(g)
    plan, db, hs = _batch([dict(st, kpoints=g["kpoints"][:4])], tables, sd)
    n_prob = len(plan.prob_n)
    H, S = hs.H.clone(), hs.S.clone()
    eig = torch.full((plan.eig_total,), -7.0, dtype=torch.float64, device=DEV)
    vec = torch.zeros_like(H)
    st_ = torch.full((n_prob,), -1, dtype=torch.int32, device=DEV)
    stream = torch.cuda.current_stream(DEV).cuda_stream
    lib = _lib.load()
    args = (n_prob, ptr(db.n), ptr(db.hs_off), ptr(db.eoff), ptr(db.order), ptr(H), ptr(S), ptr(eig), ptr(vec),
            ptr(st_))
    assert lib.skn_eigh_gen_vectors_noalloc(*args, plan.eig_total, MAX_N + 1, stream) == _lib.SKN_ERR_CAPACITY
    assert lib.skn_eigh_gen_vectors_noalloc(*args, MAX_ROWS + 1, plan.max_n, stream) == _lib.SKN_ERR_CAPACITY
    torch.cuda.synchronize(DEV)
    # nothing ran
    assert bool((eig == -7.0).all()) and bool((st_ == -1).all()) and torch.equal(H, hs.H)


def test_noalloc_zero_problem_call_is_a_warm_up():
    """A call with no problems loads the module and looks up the fixed array, and launches nothing."""
    lib = _lib.load()
    stream = torch.cuda.current_stream(DEV).cuda_stream
    assert lib.skn_eigh_gen_vectors_noalloc(0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, stream) == _lib.SKN_OK


def test_noalloc_skips_problems_past_an_understated_row_count():
    """n_rows one short of the batch's eigenvalue rows: the problem whose rows end past it is skipped on the
    device with SKN_ERR_CAPACITY and its outputs untouched; every other problem matches the allocating entry."""
    g = golden("rand_b")
    st, tables, sd = load_case(g)
    plan, db, hs = _batch([dict(st, kpoints=g["kpoints"][:6])], tables, sd)
    n_prob = len(plan.prob_n)
    eig_a, vec_a, st_a = _allocating(plan, db, hs.H, hs.S)
    H, S = hs.H.clone(), hs.S.clone()
    eig = torch.full((plan.eig_total,), -7.0, dtype=torch.float64, device=DEV)
    vec = torch.full_like(H, -3.0)
    st_ = torch.full((n_prob,), -1, dtype=torch.int32, device=DEV)
    stream = torch.cuda.current_stream(DEV).cuda_stream
    lib = _lib.load()
    rc = lib.skn_eigh_gen_vectors_noalloc(n_prob, ptr(db.n), ptr(db.hs_off), ptr(db.eoff), ptr(db.order), ptr(H),
                                          ptr(S), ptr(eig), ptr(vec), ptr(st_), plan.eig_total - 1, plan.max_n,
                                          stream)
    torch.cuda.synchronize(DEV)
    assert rc == _lib.SKN_OK
    eoff = db.eoff.cpu().tolist()
    hoff = db.hs_off.cpu().tolist()
    nv = db.n.cpu().tolist()
    status = st_.cpu().tolist()
    over = [p for p in range(n_prob) if eoff[p] + nv[p] > plan.eig_total - 1]
    assert len(over) == 1
    for p in range(n_prob):
        n = nv[p]
        e = slice(eoff[p], eoff[p] + n)
        v = slice(2 * hoff[p], 2 * (hoff[p] + n * n))    # H is held as doubles: 2 per complex entry
        if p in over:
            assert status[p] == _lib.SKN_ERR_CAPACITY
            assert bool((eig[e] == -7.0).all()) and bool((vec[v] == -3.0).all())
        else:
            assert status[p] == _lib.SKN_OK
            assert float((eig[e] - eig_a[e]).abs().max()) * EV <= 1e-8
            assert float((vec[v] - vec_a[v]).abs().max()) <= 1e-10
