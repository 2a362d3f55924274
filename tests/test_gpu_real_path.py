"""Real-arithmetic eigensolver for real H(k), S(k) (needs a GB300).

At k-points with 2k integer the Bloch phases are exactly +-1, so H(k) and S(k)
are real.  The engine sends those problems to skn_eigh_gen_batched_real, which
runs the same steps in real arithmetic.  Its eigenvalues must equal the complex
kernel's (the real path drops only terms that are exactly zero), and the golden
parity must hold with it on.
"""
import numpy as np
import pytest
import torch

from conftest import golden
from _cases import load_case
from slakonet_gb300 import engine as E, synthetic as syn

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
H2E = 27.211


def _uneven(seed, n_struct=24):
    sts = syn.uneven_batch(n_struct, nmin=2, nmax=48, zmax=65, seed=seed, kdens=300.0)
    zs = sorted({int(z) for s in sts for z in s["numbers"]})
    sd = syn.default_shell_dict()
    ts = E.TableSet.from_synthetic(syn.make_tables(zs, sd, seed=seed), {z: sd[z] for z in zs}, DEV)
    return sts, ts


def test_real_kpoints_are_marked_and_real():
    sts, ts = _uneven(3)
    plan = E.plan_batch(sts, ts)
    assert plan.prob_real.any() and (~plan.prob_real).any()
    res = E.Engine(ts).run(plan, keep_hs=True, hs_only=True)
    Hc = torch.view_as_complex(res.H.view(-1, 2))
    Sc = torch.view_as_complex(res.S.view(-1, 2))
    for p in np.nonzero(plan.prob_real)[0][:50]:
        o, n = int(plan.hs_off[p]), int(plan.prob_n[p])
        assert float(Hc[o:o + n * n].imag.abs().max()) == 0.0
        assert float(Sc[o:o + n * n].imag.abs().max()) == 0.0


@pytest.mark.parametrize("seed", [3, 5])
def test_real_path_matches_complex_kernel(seed):
    sts, ts = _uneven(seed)
    plan = E.plan_batch(sts, ts)
    a = E.Engine(ts, real_path=False).run(plan)
    b = E.Engine(ts, real_path=True).run(plan)
    assert torch.equal(a.eig_status, b.eig_status)
    de = float((a.eig - b.eig).abs().max()) * H2E
    same = torch.equal(a.eig, b.eig)
    print(f"seed {seed}: {int(plan.prob_real.sum())} of {len(plan.prob_n)} problems real; "
          f"max |de| {de:.1e} eV, bitwise {same}")
    assert de <= 1e-12


def test_real_path_golden_gamma_centred_cell():
    """rand_c's golden Gamma-centred grid contains real k-points; parity holds with the real path."""
    g = golden("rand_c")
    st, tables, sd = load_case(g)
    ts = E.TableSet.from_synthetic(tables, sd, DEV)
    s = {"numbers": st["numbers"], "positions": st["positions"], "cell": st["cell"], "kpoints": g["kpoints"],
         "weights": g["k_weights"]}
    plan = E.plan_batch([s], ts)
    assert plan.prob_real.any()
    res = E.Engine(ts, real_path=True).run(plan)
    de = np.abs(res.eigenvalues(0).cpu().numpy() - g["eigenvalues"]).max() * H2E
    print(f"rand_c: {int(plan.prob_real.sum())} real k-points, eig error {de:.1e} eV")
    assert de <= 1e-8
