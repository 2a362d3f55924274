"""Eigenvectors of the CUDA path (needs a GB300).

Checks per (structure, k): residual ||H C - S C diag(e)|| / ||H|| <= 1e-10,
S-orthonormality ||C^H S C - I|| <= 1e-10, and for well-separated bands the
direction agrees with the oracle's eigh (|c^H S c_oracle| = 1 within 1e-8).
"""
import numpy as np
import pytest
import torch

from conftest import golden
from _cases import load_case
from oracle import slako_oracle as O
from slakonet_gb300 import engine as E, model as M, synthetic as syn

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _check(st, tables, sd, k):
    ts = E.TableSet.from_synthetic(tables, sd, DEV)
    plan = E.plan_batch([dict(st, kpoints=k)], ts)
    eng = E.Engine(ts)
    hs = eng.run(plan, keep_hs=True, hs_only=True)
    res = eng.run(plan, vectors=True)
    n = int(plan.nb[0])
    H = torch.view_as_complex(hs.H.view(-1, 2)).view(len(k), n, n).transpose(1, 2).cpu().numpy()
    S = torch.view_as_complex(hs.S.view(-1, 2)).view(len(k), n, n).transpose(1, 2).cpu().numpy()
    C = res.eigenvectors(0).cpu().numpy()
    e = res.eigenvalues(0).cpu().numpy()
    worst_r = worst_o = worst_d = 0.0
    for q in range(len(k)):
        Hq, Sq, Cq = H[q], S[q], C[q]
        r = np.abs(Hq @ Cq - Sq @ Cq * e[q][None, :]).max() / np.abs(Hq).max()
        o = np.abs(Cq.conj().T @ Sq @ Cq - np.eye(n)).max()
        worst_r, worst_o = max(worst_r, r), max(worst_o, o)
        w_ref, v_ref = O.eigh_generalized(Hq, Sq, vectors=True)
        gaps = np.diff(w_ref)
        iso = np.ones(n, bool)
        iso[:-1] &= gaps > 1e-6
        iso[1:] &= gaps > 1e-6
        ov = np.abs(np.einsum("ij,ik,kj->j", Cq.conj(), Sq, v_ref))
        if iso.any():
            worst_d = max(worst_d, np.abs(ov[iso] - 1.0).max())
    return worst_r, worst_o, worst_d


@pytest.mark.parametrize("case", ["si_cfg0", "rand_f4", "rand_b", "rand_c"])
def test_eigenvectors_against_oracle(case):
    g = golden(case)
    st, tables, sd = load_case(g)
    k = g["kpoints"]
    k = k[np.linspace(0, len(k) - 1, min(len(k), 12)).astype(int)]
    r, o, d = _check(st, tables, sd, k)
    print(f"{case}: residual {r:.1e}, orthonormality {o:.1e}, direction {d:.1e}")
    assert r <= 1e-10 and o <= 1e-10 and d <= 1e-8


def test_eigenvectors_degenerate_diamond_gamma():
    """Gamma and high-symmetry points of diamond Si carry exactly degenerate bands."""
    g = golden("si_cfg0")
    st, tables, sd = load_case(g)
    k = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.0], [0.5, 0.0, 0.0], [0.25, 0.25, 0.25]])
    r, o, d = _check(st, tables, sd, k)
    print(f"degenerate: residual {r:.1e}, orthonormality {o:.1e}")
    assert r <= 1e-10 and o <= 1e-10


def test_with_eigenvectors_drop_in_layout():
    g = golden("si_cfg0")
    st, tables, sd = load_case(g)
    model = M.MultiElementSkfParameterOptimizer.from_tables(tables)
    geom = M.Geometry(st["numbers"], st["positions"], st["cell"])
    props, ok = model.compute_multi_element_properties(geometry=geom, shell_dict=sd, kpoints=torch.tensor([2, 2, 2]),
                                                       get_fermi=True, device=DEV, with_eigenvectors=True)
    ev = props["calc"].eigenvectors
    assert ev.shape == (1, 18, 18, 8) and ev.dtype == torch.complex128


def test_eigenvectors_finite_where_the_eigenvalue_is_exact():
    """A 5-atom cell of the 64-structure fitting batch (n = 35, 200 k-points) whose eigenvalues the Sturm/Newton
    step finds to the last bit at some k-points: T - e I then has a zero pivot, and inverse iteration must still
    return finite, S-orthonormal eigenvectors (with a 1e-300 pivot floor one solve overflowed to NaN)."""
    from slakonet_gb300 import training as T
    batch = T.fitting_batch(64, seed=0)
    st = batch[38]
    sd = syn.default_shell_dict()
    zs = sorted({int(z) for s in batch for z in s["numbers"]})     # the batch's tables (one seeded draw)
    tables = syn.make_tables(zs, sd, seed=0)
    sdz = {z: sd[z] for z in zs}
    ts = E.TableSet.from_synthetic(tables, sdz, DEV)
    plan = E.plan_batch([st], ts)
    res = E.Engine(ts).run(plan, vectors=True)
    C = res.eigenvectors(0)
    assert bool(torch.isfinite(torch.view_as_real(C)).all())
    k = np.asarray(st["kpoints"])
    sub = {key: v for key, v in st.items() if key != "weights"}      # _check sets its own k-points
    r, o, d = _check(sub, tables, sdz, k[np.linspace(0, len(k) - 1, 24).astype(int)])
    print(f"fitting-batch cell (n = {int(plan.nb[0])}, {len(k)} k): all {len(k)} k-points finite; "
          f"residual {r:.1e}, orthonormality {o:.1e}, direction {d:.1e}")
    assert r <= 1e-10 and o <= 1e-10 and d <= 1e-8
