"""Hand-written adjoint vs the reference's autograd (conjugate restored) and central differences.

Gate: parameter gradients within 1e-8 relative (max abs error / max abs
entry) of the reference's autograd with the eigenvector conjugate restored;
central differences (h = 1e-5, with one Richardson step against h/2 to remove
the O(h^2) truncation that 0.1 eV Gaussians make visible) within 1e-6
relative for a DOS + gap loss with the Fermi level held fixed.
The reference's shipped autograd, which drops that conjugate, disagrees with
both; the fixtures record it and the test reports the disagreement.
"""
import numpy as np
import pytest
import torch

from conftest import golden
from _cases import tables_checksum
from slakonet_gb300 import adjoint as A, model as M, synthetic as syn

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _load(name):
    g = golden(name)
    st = {"numbers": g["numbers"], "positions": g["positions"], "cell": g["cell"]}
    if "shells" in g.files:
        sd = {14: [int(x) for x in g["shells"]]}
        tables = syn.make_tables([14], sd, seed=int(g["seed"]))
    else:
        full = syn.default_shell_dict()
        tables = syn.make_tables(st["numbers"], full, seed=int(g["table_seed"]))
        sd = {int(z): full[int(z)] for z in st["numbers"]}
    np.testing.assert_allclose(tables_checksum(tables), g["tables_checksum"], rtol=1e-12, atol=1e-300)
    return g, st, tables, sd


@pytest.mark.parametrize("name", ["grad_si", "grad_hetero"])
def test_adjoint_matches_reference_autograd(name):
    g, st, tables, sd = _load(name)
    model = M.MultiElementSkfParameterOptimizer.from_tables(tables)
    k = g["kpoints"]
    s = dict(st, kpoints=k, weights=np.full(len(k), 1.0 / len(k)))
    eig, dos, gap, res = A.differentiable_properties(model, [s], sd, DEV)
    loss = torch.sin(5.0 * eig + 0.3).sum()
    assert abs(loss.item() - float(g["loss"])) <= 1e-9 * max(1.0, abs(float(g["loss"])))
    loss.backward()
    worst, worst_ship, scale = 0.0, 0.0, 0.0
    for key in [k_[len("fixed|"):] for k_ in g.files if k_.startswith("fixed|")]:
        pair, kind, lk = key.split("|")
        prm = getattr(model.skf_optimizers[pair], f"{kind}_params")[lk]
        ours = prm.grad.detach().cpu().numpy() if prm.grad is not None else np.zeros(prm.shape)
        ref = g["fixed|" + key]
        worst = max(worst, np.abs(ours - ref).max())
        worst_ship = max(worst_ship, np.abs(ours - g["shipped|" + key]).max())
        scale = max(scale, np.abs(ref).max())
    print(f"{name}: adjoint vs corrected reference autograd {worst / scale:.1e} rel; "
          f"vs shipped reference autograd {worst_ship / scale:.1e} rel")
    assert worst <= 1e-8 * scale
    # the fixture's central differences agree with the corrected gradient
    for (key, idx, vals) in zip(g["fd_keys"], g["fd_idx"], g["fd_values"]):
        assert abs(vals[0] - vals[1]) <= 1e-5 * abs(vals[0])


def _dos_torch(eig_flat, res, s, mu):
    """Gaussian DOS of structure s from eigenvalues (torch autograd), Fermi level held at mu."""
    plan = res.plan
    o, nk, nb = int(plan.eig_off_struct[s]), int(plan.nk[s]), int(plan.nb[s])
    e = ((eig_flat[o:o + nk * nb].view(nk, nb) - mu) * 27.211)
    w = torch.as_tensor(plan.kweights[plan.k_ptr[s]:plan.k_ptr[s + 1]], device=eig_flat.device)
    grid = res.dos_grid
    x = (grid[None, None, :] - e[:, :, None]) / 0.1
    g = torch.exp(-0.5 * x * x) / (0.1 * np.sqrt(2 * np.pi))
    return (w[:, None, None] * g).sum((0, 1))


def test_dos_backward_kernel_matches_autograd_of_the_dos_formula():
    g, st, tables, sd = _load("grad_hetero")
    model = M.MultiElementSkfParameterOptimizer.from_tables(tables)
    k = syn.gamma_centred_kpoints((2, 2, 1))
    s = dict(st, kpoints=k, weights=np.full(len(k), 1.0 / len(k)))
    c = torch.as_tensor(np.random.default_rng(5).standard_normal(1000), device=DEV)
    eig, dos, gap, res = A.differentiable_properties(model, [s], sd, DEV, dos_window=0.0)
    (dos[0] * c).sum().backward()
    ga = {n: p.grad.clone() for n, p in model.named_parameters() if p.grad is not None}
    model.zero_grad()
    eig, dos, gap, res = A.differentiable_properties(model, [s], sd, DEV, dos_window=0.0)
    mu = float(res.mu[0])
    (_dos_torch(eig, res, 0, mu) * c).sum().backward()
    gb = {n: p.grad.clone() for n, p in model.named_parameters() if p.grad is not None}
    scale = max(float(v.abs().max()) for v in gb.values())
    worst = max(float((ga[n] - gb[n]).abs().max()) for n in gb)
    print(f"DOS backward kernel vs autograd of the DOS formula: {worst / scale:.1e} rel")
    assert worst <= 1e-10 * scale


def test_adjoint_dos_gap_loss_against_finite_differences():
    """Loss = DOS MSE + |gap - 1|, Fermi level held fixed (the reference detaches it)."""
    g, st, tables, sd = _load("grad_hetero")
    model = M.MultiElementSkfParameterOptimizer.from_tables(tables)
    k = syn.gamma_centred_kpoints((2, 2, 1))
    s = dict(st, kpoints=k, weights=np.full(len(k), 1.0 / len(k)))
    rng = np.random.default_rng(3)
    target = torch.as_tensor(rng.uniform(0, 2, 1000), device=DEV)
    _, _, _, res0 = A.differentiable_properties(model, [s], sd, DEV)
    mu0 = float(res0.mu[0])

    def loss_fn():
        eig, dos, gap, res = A.differentiable_properties(model, [s], sd, DEV)
        return ((_dos_torch(eig, res, 0, mu0) - target) ** 2).mean() + (gap[0] - 1.0).abs()

    loss = loss_fn()
    loss.backward()
    checked = 0
    worst = worst_plain = 0.0
    prm_list = [getattr(opt, f"{kind}_params")[lk] for key, opt in model.skf_optimizers.items()
                for kind in ("h", "s") for lk in getattr(opt, f"{kind}_params")]
    for prm in prm_list:
        gr = prm.grad
        if gr is None or float(gr.abs().max()) == 0.0:
            continue
        idx = np.unravel_index(int(torch.argmax(gr.abs())), gr.shape)
        def central(h):
            with torch.no_grad():
                old = float(prm[idx])
                prm[idx] = old + h
                lp = float(loss_fn())
                prm[idx] = old - h
                lm = float(loss_fn())
                prm[idx] = old
            return (lp - lm) / (2 * h)

        fd1 = central(1e-5)
        fd2 = central(0.5e-5)
        rich = (4.0 * fd2 - fd1) / 3.0        # removes the O(h^2) truncation term
        an = float(gr[idx])
        worst = max(worst, abs(rich - an) / max(abs(rich), 1e-12))
        worst_plain = max(worst_plain, abs(fd1 - an) / max(abs(fd1), 1e-12))
        checked += 1
        if checked >= 6:
            break
    print(f"DOS+gap loss: {checked} entries, |FD(h=1e-5) - adjoint| / |FD| <= {worst_plain:.1e}, "
          f"Richardson(h=1e-5, 5e-6) {worst:.1e}")
    assert checked >= 3 and worst <= 1e-6
