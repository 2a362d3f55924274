"""Cluster eigensolver (one thread-block cluster per problem) on a GB300.

Eigenvalues from skn_eigh_gen_large must agree with the one-CTA-per-problem
eigensolver and with the oracle within 1e-8 eV at every cluster size, the
engine's routing of large problems must leave the golden results unchanged,
and problems above the one-CTA bound (n > 2048) are checked against LAPACK
(scipy) in FP64.
"""
import ctypes

import numpy as np
import pytest
import scipy.linalg as sla
import torch

from conftest import golden
from _cases import load_case
from slakonet_gb300 import engine as E, synthetic as syn
from slakonet_gb300._lib import SknError, call, ptr

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
H2E = 27.211


def _problems(sizes, seed, spd=True):
    """Random Hermitian H and Hermitian positive definite S (column-major per problem)."""
    rng = np.random.default_rng(seed)
    Hs, Ss = [], []
    for n in sizes:
        X = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        H = (X + X.conj().T) / 2
        Y = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * 0.1
        S = np.eye(n) + Y @ Y.conj().T / n
        if not spd:
            S = S - 2.0 * np.eye(n)
        Hs.append(H)
        Ss.append(S)
    return Hs, Ss


def _pack(mats):
    flat = np.concatenate([m.T.reshape(-1) for m in mats])      # column-major
    return torch.as_tensor(np.stack([flat.real, flat.imag], 1).reshape(-1), device=DEV)


def _solve(Hs, Ss, cluster=None):
    """Eigenvalues per problem from the cluster kernel (cluster = CTAs) or the one-CTA kernel (None)."""
    sizes = np.array([h.shape[0] for h in Hs])
    n_prob = len(sizes)
    hs_off = np.concatenate([[0], np.cumsum(sizes.astype(np.int64) ** 2)[:-1]])
    eoff = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    order = np.argsort(-sizes, kind="stable").astype(np.int32)
    nv = torch.as_tensor(sizes.astype(np.int32), device=DEV)
    off = torch.as_tensor(hs_off, device=DEV)
    eo = torch.as_tensor(eoff, device=DEV)
    od = torch.as_tensor(order, device=DEV)
    H, S = _pack(Hs), _pack(Ss)
    eig = torch.empty(int(sizes.sum()), dtype=torch.float64, device=DEV)
    st = torch.empty(n_prob, dtype=torch.int32, device=DEV)
    ctr = torch.zeros(2, dtype=torch.int32, device=DEV)
    stream = torch.cuda.current_stream(DEV).cuda_stream
    max_n = int(sizes.max())
    if cluster is None:
        call("skn_eigh_gen_batched", n_prob, ptr(nv), ptr(off), ptr(eo), ptr(od), ptr(H), ptr(S), ptr(eig), ptr(st),
             ptr(ctr), max_n, stream)
    else:
        need = ctypes.c_int64(0)
        call("skn_eigh_large_scratch_bytes", n_prob, max_n, cluster, ctypes.addressof(need))
        scratch = torch.empty(need.value // 8, dtype=torch.float64, device=DEV)
        call("skn_eigh_gen_large", n_prob, ptr(nv), ptr(off), ptr(eo), ptr(od), ptr(H), ptr(S), ptr(eig), ptr(st),
             ptr(ctr), ptr(scratch), need.value, max_n, cluster, stream)
    torch.cuda.synchronize(DEV)
    e = eig.cpu().numpy()
    return [e[eoff[p]:eoff[p] + sizes[p]] for p in range(n_prob)], st.cpu().numpy()


@pytest.mark.parametrize("cluster", [1, 2, 3, 4, 8, 12, 16])
def test_cluster_sizes_agree_with_single_cta_and_lapack(cluster):
    sizes = [1, 2, 7, 33, 130, 257, 301]   # odd largest n: per-cluster scratch alignment
    Hs, Ss = _problems(sizes, seed=cluster)
    ref, st_ref = _solve(Hs, Ss)
    got, st = _solve(Hs, Ss, cluster)
    assert (st == 0).all() and (st_ref == 0).all()
    d_single = max(np.abs(a - b).max() for a, b in zip(got, ref)) * H2E
    d_lapack = max(np.abs(a - sla.eigh(h, s, eigvals_only=True)).max() for a, h, s in zip(got, Hs, Ss)) * H2E
    print(f"cluster {cluster}: vs one-CTA kernel {d_single:.1e} eV, vs LAPACK {d_lapack:.1e} eV")
    assert d_single <= 1e-8 and d_lapack <= 1e-8


def test_problems_above_the_single_cta_bound():
    """n = 2500 and 3000 (H, S 100-144 MB each): one 16-CTA cluster per problem vs LAPACK."""
    Hs, Ss = _problems([2500, 3000], seed=7)
    got, st = _solve(Hs, Ss, 16)
    assert (st == 0).all()
    worst = 0.0
    for a, h, s in zip(got, Hs, Ss):
        ref = sla.eigh(h, s, eigvals_only=True)
        worst = max(worst, np.abs(a - ref).max() / max(1.0, np.abs(ref).max()))
    print(f"n = 2500, 3000: max |de| / max(1, |e|max) = {worst:.1e}")
    assert worst * H2E <= 1e-8


def test_not_positive_definite_overlap_reported_by_cluster_path():
    Hs, Ss = _problems([40, 90], seed=3, spd=False)
    got, st = _solve(Hs, Ss, 4)
    assert (st == 2).all()
    assert all(np.isnan(g).all() for g in got)


@pytest.mark.parametrize("case", ["si_cfg0", "rand_b"])
def test_engine_cluster_route_matches_golden(case):
    """large_threshold = 0 sends every problem of the golden case through the cluster path."""
    g = golden(case)
    st, tables, sd = load_case(g)
    ts = E.TableSet.from_synthetic(tables, sd, DEV)
    s = {"numbers": st["numbers"], "positions": st["positions"], "cell": st["cell"], "kpoints": g["kpoints"],
         "weights": g["k_weights"]}
    for cluster in (2, 16):
        res = E.Engine(ts, large_threshold=0, large_cluster=cluster).run(E.plan_batch([s], ts))
        assert (res.eig_status.cpu().numpy() == 0).all()
        de = np.abs(res.eigenvalues(0).cpu().numpy() - g["eigenvalues"]).max() * H2E
        dmu = abs(float(res.mu[0]) * H2E - float(g["fermi_energy_eV"]))
        print(f"{case}, cluster {cluster}: eig {de:.1e} eV, E_F {dmu:.1e} eV")
        assert de <= 1e-8 and dmu <= 1e-6


def test_engine_mixed_batch_split_between_kernels():
    """Problems above 100 orbitals on the cluster path, the rest on the one-CTA path, concurrently."""
    sts = syn.uneven_batch(10, nmin=2, nmax=40, zmax=30, seed=4, kdens=100.0)
    zs = sorted({int(z) for x in sts for z in x["numbers"]})
    sd = syn.default_shell_dict()
    ts = E.TableSet.from_synthetic(syn.make_tables(zs, sd, seed=4), {z: sd[z] for z in zs}, DEV)
    plan = E.plan_batch(sts, ts)
    assert (plan.prob_n > 100).any() and (plan.prob_n <= 100).any()
    a = E.Engine(ts, large_threshold=None).run(plan)
    b = E.Engine(ts, large_threshold=100, large_cluster=8).run(plan)
    assert (b.eig_status.cpu().numpy() == 0).all()
    de = float((a.eig - b.eig).abs().max()) * H2E
    small = torch.as_tensor(np.repeat(plan.prob_n <= 100, plan.prob_n), device=DEV)
    print(f"mixed batch: max |de| {de:.1e} eV over {len(plan.prob_n)} problems")
    assert de <= 1e-8
    assert torch.equal(a.eig[small], b.eig[small])   # the one-CTA problems are untouched


def test_capacity_errors():
    with pytest.raises(SknError):
        need = ctypes.c_int64(0)
        call("skn_eigh_large_scratch_bytes", 1, 9217, 16, ctypes.addressof(need))
    with pytest.raises(SknError):
        call("skn_eigh_large_scratch_bytes", 1, 100, 17, ctypes.addressof(ctypes.c_int64(0)))
