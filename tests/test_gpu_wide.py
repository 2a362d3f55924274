"""Device-wide eigensolver (csrc/eigh_wide.cu) on a GB300.

skn_eigh_gen_wide must agree with LAPACK (scipy) and with the one-CTA kernel within 1e-8 eV on
random Hermitian-definite pairs, including sizes that leave partial panels and tiles; give the
same results in real arithmetic on real problems; report a non-positive-definite S(k) as
SKN_ERR_NOT_SPD with NaN eigenvalues without disturbing the other problems of its group; give a
problem bitwise the same eigenvalues alone and in a group; and, routed by the engine, leave the
golden cases' results unchanged.
"""
import ctypes

import numpy as np
import pytest
import scipy.linalg as sla
import torch

from conftest import golden
from _cases import load_case
from slakonet_gb300 import engine as E, synthetic as syn
from slakonet_gb300._lib import call, ptr

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
H2E = 27.211


def _pairs(n, count, seed, real=False, spd=True):
    rng = np.random.default_rng(seed)
    Hs, Ss = [], []
    for _ in range(count):
        X = rng.standard_normal((n, n)) + (0 if real else 1j) * rng.standard_normal((n, n))
        H = (X + X.conj().T) / 2
        Y = (rng.standard_normal((n, n)) + (0 if real else 1j) * rng.standard_normal((n, n))) * 0.1
        S = np.eye(n) + Y @ Y.conj().T / n
        if not spd:
            S = S - 2.0 * np.eye(n)
        Hs.append(H.astype(np.complex128))
        Ss.append(S.astype(np.complex128))
    return Hs, Ss


def _pack(mats):
    flat = np.concatenate([m.T.reshape(-1) for m in mats])      # column-major
    return torch.as_tensor(np.stack([flat.real, flat.imag], 1).reshape(-1), device=DEV)


def _wide(Hs, Ss, real=False, slots=None):
    """Eigenvalues from skn_eigh_gen_wide; `slots` reorders the group (problem index per slot)."""
    n = Hs[0].shape[0]
    count = len(Hs)
    nv = torch.full((count,), n, dtype=torch.int32, device=DEV)
    off = torch.arange(count, dtype=torch.int64, device=DEV) * n * n
    eo = torch.arange(count, dtype=torch.int64, device=DEV) * n
    prob = torch.as_tensor(np.arange(count) if slots is None else np.asarray(slots), dtype=torch.int32, device=DEV)
    H, S = _pack(Hs), _pack(Ss)
    eig = torch.full((count * n,), -7.0, dtype=torch.float64, device=DEV)
    st = torch.full((count,), -1, dtype=torch.int32, device=DEV)
    need = ctypes.c_int64(0)
    call("skn_eigh_wide_scratch_bytes", len(prob), n, ctypes.addressof(need))
    scratch = torch.empty(need.value // 8, dtype=torch.float64, device=DEV)
    call("skn_eigh_gen_wide", len(prob), n, ptr(prob), ptr(nv), ptr(off), ptr(eo), ptr(H), ptr(S), ptr(eig), ptr(st),
         ptr(scratch), need.value, int(real), torch.cuda.current_stream(DEV).cuda_stream)
    torch.cuda.synchronize(DEV)
    return eig.cpu().numpy().reshape(count, n), st.cpu().numpy()


def _single(Hs, Ss):
    n = Hs[0].shape[0]
    count = len(Hs)
    nv = torch.full((count,), n, dtype=torch.int32, device=DEV)
    off = torch.arange(count, dtype=torch.int64, device=DEV) * n * n
    eo = torch.arange(count, dtype=torch.int64, device=DEV) * n
    order = torch.arange(count, dtype=torch.int32, device=DEV)
    H, S = _pack(Hs), _pack(Ss)
    eig = torch.empty(count * n, dtype=torch.float64, device=DEV)
    st = torch.empty(count, dtype=torch.int32, device=DEV)
    ctr = torch.zeros(2, dtype=torch.int32, device=DEV)
    call("skn_eigh_gen_batched", count, ptr(nv), ptr(off), ptr(eo), ptr(order), ptr(H), ptr(S), ptr(eig), ptr(st),
         ptr(ctr), n, torch.cuda.current_stream(DEV).cuda_stream)
    torch.cuda.synchronize(DEV)
    return eig.cpu().numpy().reshape(count, n), st.cpu().numpy()


@pytest.mark.parametrize("n", [1, 2, 31, 33, 64, 65, 100, 257, 700])
def test_wide_agrees_with_lapack_and_single_cta(n):
    Hs, Ss = _pairs(n, 3, seed=n)
    got, st = _wide(Hs, Ss)
    ref, st_ref = _single(Hs, Ss)
    assert (st == 0).all() and (st_ref == 0).all()
    d_lapack = max(np.abs(got[i] - sla.eigh(Hs[i], Ss[i], eigvals_only=True)).max() for i in range(3)) * H2E
    d_single = np.abs(got - ref).max() * H2E
    print(f"n = {n}: vs LAPACK {d_lapack:.1e} eV, vs one-CTA kernel {d_single:.1e} eV")
    assert d_lapack <= 1e-8 and d_single <= 1e-8


@pytest.mark.parametrize("n", [70, 300])
def test_real_arithmetic_on_real_problems(n):
    Hs, Ss = _pairs(n, 2, seed=100 + n, real=True)
    a, sa = _wide(Hs, Ss, real=False)
    b, sb = _wide(Hs, Ss, real=True)
    assert (sa == 0).all() and (sb == 0).all()
    ref = np.stack([sla.eigh(Hs[i].real, Ss[i].real, eigvals_only=True) for i in range(2)])
    print(f"n = {n}: real vs complex arithmetic {np.abs(a - b).max() * H2E:.1e} eV, "
          f"real vs LAPACK {np.abs(b - ref).max() * H2E:.1e} eV, bitwise equal: {np.array_equal(a, b)}")
    assert np.abs(a - b).max() * H2E <= 1e-8 and np.abs(b - ref).max() * H2E <= 1e-8


def test_not_positive_definite_problem_alone_in_its_group():
    Hs, Ss = _pairs(90, 3, seed=5)
    bad_H, bad_S = _pairs(90, 1, seed=6, spd=False)
    Hs[1], Ss[1] = bad_H[0], bad_S[0]
    got, st = _wide(Hs, Ss)
    assert st.tolist() == [0, 2, 0]
    assert np.isnan(got[1]).all()
    for i in (0, 2):
        assert np.abs(got[i] - sla.eigh(Hs[i], Ss[i], eigvals_only=True)).max() * H2E <= 1e-8


def test_results_do_not_depend_on_the_group():
    Hs, Ss = _pairs(150, 4, seed=9)
    together, _ = _wide(Hs, Ss, slots=[3, 1, 0, 2])
    for i in range(4):
        alone, st = _wide([Hs[i]], [Ss[i]])
        assert st[0] == 0
        assert np.array_equal(alone[0], together[i]), i


def test_size_mismatch_is_refused_per_problem():
    """A slot whose problem has another size gets SKN_ERR_CAPACITY and its eigenvalues untouched."""
    Hs, Ss = _pairs(40, 2, seed=11)
    n = 40
    nv = torch.tensor([n, n + 1], dtype=torch.int32, device=DEV)
    off = torch.tensor([0, n * n], dtype=torch.int64, device=DEV)
    eo = torch.tensor([0, n], dtype=torch.int64, device=DEV)
    prob = torch.tensor([0, 1], dtype=torch.int32, device=DEV)
    H, S = _pack(Hs), _pack(Ss)
    eig = torch.full((2 * n,), -7.0, dtype=torch.float64, device=DEV)
    st = torch.full((2,), -1, dtype=torch.int32, device=DEV)
    need = ctypes.c_int64(0)
    call("skn_eigh_wide_scratch_bytes", 2, n, ctypes.addressof(need))
    scratch = torch.empty(need.value // 8, dtype=torch.float64, device=DEV)
    call("skn_eigh_gen_wide", 2, n, ptr(prob), ptr(nv), ptr(off), ptr(eo), ptr(H), ptr(S), ptr(eig), ptr(st),
         ptr(scratch), need.value, 0, torch.cuda.current_stream(DEV).cuda_stream)
    torch.cuda.synchronize(DEV)
    assert st.cpu().tolist() == [0, 5]
    assert (eig[n:] == -7.0).all()


@pytest.mark.parametrize("case", ["si_cfg0", "rand_b"])
def test_engine_routing_to_the_wide_path_keeps_golden_results(case):
    """wide_threshold = 0 sends every problem of the golden case through the device-wide path."""
    g = golden(case)
    st, tables, sd = load_case(g)
    ts = E.TableSet.from_synthetic(tables, sd, DEV)
    s = {"numbers": st["numbers"], "positions": st["positions"], "cell": st["cell"], "kpoints": g["kpoints"],
         "weights": g["k_weights"]}
    res = E.Engine(ts, large_threshold=None, wide_threshold=0).run(E.plan_batch([s], ts))
    assert (res.eig_status.cpu().numpy() == 0).all()
    de = np.abs(res.eigenvalues(0).cpu().numpy() - g["eigenvalues"]).max() * H2E
    dmu = abs(float(res.mu[0]) * H2E - float(g["fermi_energy_eV"]))
    print(f"{case}, wide path: eig {de:.1e} eV, E_F {dmu:.1e} eV")
    assert de <= 1e-8 and dmu <= 1e-6


def test_engine_mixed_batch_split_between_wide_and_single_cta():
    """Problems above 100 orbitals on the wide path (one group per size, on side streams), the rest
    on the one-CTA path; the one-CTA problems' results are bitwise unchanged."""
    sts = syn.uneven_batch(10, nmin=2, nmax=40, zmax=30, seed=4, kdens=100.0)
    zs = sorted({int(z) for x in sts for z in x["numbers"]})
    sd = syn.default_shell_dict()
    ts = E.TableSet.from_synthetic(syn.make_tables(zs, sd, seed=4), {z: sd[z] for z in zs}, DEV)
    plan = E.plan_batch(sts, ts)
    assert (plan.prob_n > 100).any() and (plan.prob_n <= 100).any()
    a = E.Engine(ts, large_threshold=None).run(plan)
    b = E.Engine(ts, large_threshold=None, wide_threshold=100).run(plan)
    assert (b.eig_status.cpu().numpy() == 0).all()
    de = float((a.eig - b.eig).abs().max()) * H2E
    small = torch.as_tensor(np.repeat(plan.prob_n <= 100, plan.prob_n), device=DEV)
    print(f"mixed batch, wide path above 100 orbitals: max |de| {de:.1e} eV over {len(plan.prob_n)} problems")
    assert de <= 1e-8
    assert torch.equal(a.eig[small], b.eig[small])
