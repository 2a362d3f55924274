"""CUDA path vs the reference's golden outputs and the CPU oracle (needs a GB300).

Tolerances (stated by the task and checked here, each measured error printed):
H(k)/S(k) <= 1e-12 relative (max abs error / max abs entry), eigenvalues
<= 1e-8 eV, DOS <= 1e-6 max-abs, Fermi level and gap <= 1e-6 eV.
"""
import numpy as np
import pytest
import torch

from conftest import golden
from _cases import CASES, load_case
from oracle import slako_oracle as O
from slakonet_gb300 import engine as E, model as M, synthetic as syn

pytestmark = pytest.mark.gpu
H2E = 27.211
DEV = "cuda:0"


def _tables(tables, sd):
    return E.TableSet.from_synthetic(tables, sd, DEV)


def _struct(st, k, w=None):
    d = {"numbers": st["numbers"], "positions": st["positions"], "cell": st["cell"], "kpoints": k}
    if w is not None:
        d["weights"] = w
    return d


def _hs(res, s, plan):
    p = np.nonzero(plan.prob_struct == s)[0]
    n = int(plan.nb[s])
    H = res.H.view(-1, 2).cpu().numpy()
    S = res.S.view(-1, 2).cpu().numpy()
    out = []
    for M_ in (H, S):
        mats = []
        for q in p:
            o = int(plan.hs_off[q])
            a = M_[o:o + n * n]
            mats.append((a[:, 0] + 1j * a[:, 1]).reshape(n, n).T)   # column-major
        out.append(np.array(mats))
    return out


def test_spline_through_bloch_sum_matches_reference_interpolation():
    """s-s dimers at the golden distances: H(Gamma)[0,1] is the interpolated table value."""
    g = golden("interp")
    tab, r, vals = g["table"], g["r"], g["values"]
    row = tab[0:1]
    tables = {"grid": syn.grid_points(), "step": float(g["step"]),
              "elements": {1: {"shells": [0], "on_sites": np.array([0.1]), "occupations": np.array([1.0])}},
              "pairs": {(1, 1): {"H": {(0, 0): row}, "S": {(0, 0): 0.5 * row}}}}
    ts = _tables(tables, {1: [0]})
    L = 60.0
    sts = []
    for ri in r:
        sts.append({"numbers": np.array([1, 1]), "positions": np.array([[1.0, 1.0, 1.0], [1.0 + ri, 1.0, 1.0]]),
                    "cell": np.eye(3) * L, "kpoints": np.zeros((1, 3))})
    eng = E.Engine(ts, cutoff=16.0)
    res = eng.run(E.plan_batch(sts, ts, 16.0), keep_hs=True, hs_only=True)
    got = np.array([_hs(res, s, res.plan)[0][0][0, 1].real for s in range(len(sts))])
    ref = vals[:, 0]
    err = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)
    inside = r < (len(tables["grid"]) - 1) * 0.02
    print("spline rel err: grid %.2e, tail %.2e" % (err[inside].max(), err[~inside].max() if (~inside).any() else 0))
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("case", CASES)
def test_hk_sk_match_reference(case):
    g = golden(case)
    if "hk" not in g.files:
        pytest.skip("no H(k) in fixture")
    st, tables, sd = load_case(g)
    ts = _tables(tables, sd)
    k = g["kpoints"][g["hs_kindex"]]
    res = E.Engine(ts).run(E.plan_batch([_struct(st, k)], ts), keep_hs=True, hs_only=True)
    H, S = _hs(res, 0, res.plan)
    eh = np.abs(H - g["hk"]).max() / np.abs(g["hk"]).max()
    es = np.abs(S - g["sk"]).max() / np.abs(g["sk"]).max()
    print(f"{case}: H rel err {eh:.2e}, S rel err {es:.2e}")
    assert eh <= 1e-12 and es <= 1e-12


@pytest.mark.parametrize("case", CASES)
def test_eigenvalues_and_properties_match_reference(case):
    g = golden(case)
    st, tables, sd = load_case(g)
    ts = _tables(tables, sd)
    k, w = g["kpoints"], g["k_weights"]
    res = E.Engine(ts).run(E.plan_batch([_struct(st, k, w)], ts))
    assert (res.eig_status.cpu().numpy() == 0).all()
    eig = res.eigenvalues(0).cpu().numpy()
    de = np.abs(eig - g["eigenvalues"]).max() * H2E
    p = M.properties_dict(res, 0, get_fermi=True)
    dmu = abs(p["fermi_energy_eV"] - float(g["fermi_energy_eV"]))
    dgap = abs(float(p["band_gap_eV"]) - float(g["band_gap_eV"]))
    ddos = np.abs(p["dos_values_tensor"].cpu().numpy() - g["dos_values"]).max()
    print(f"{case}: eig {de:.2e} eV, E_F {dmu:.2e} eV, gap {dgap:.2e} eV, DOS {ddos:.2e}")
    assert de <= 1e-8
    assert dmu <= 1e-6 and dgap <= 1e-6 and ddos <= 1e-6
    np.testing.assert_array_equal(p["dos_energy_grid_tensor"].cpu().numpy(), g["dos_energy_grid"])
    assert abs(p["efermi"].item() - float(g["efermi_eV"])) <= 1e-6
    assert abs(p["bandgap"].item() - float(g["bandgap_eV"])) <= 1e-6
    for key in ("vbm_eV", "cbm_eV", "valence_band_width_eV", "conduction_band_width_eV", "dos_at_fermi",
                "dos_gap_center_eV", "dos_total_states"):
        assert abs(p[key] - float(g[key])) <= 1e-6, key
    # VBM/CBM k-points: symmetry-equivalent k-points carry equal band edges up to rounding, so the
    # reported index must hold the reference's band edge (within 1e-6 eV), not be the same index
    ref_e = g["eigenvalues"] * H2E
    metal = np.abs(ref_e - float(g["fermi_energy_eV"])).min() < 1e-3
    if metal:   # the reference reports E_F at k-point 0 for both edges
        assert p["vbm_kpoint"] == 0 and p["cbm_kpoint"] == 0
    else:
        assert np.abs(ref_e[p["vbm_kpoint"]] - float(g["vbm_eV"])).min() <= 1e-6
        assert np.abs(ref_e[p["cbm_kpoint"]] - float(g["cbm_eV"])).min() <= 1e-6
    if p["vbm_kpoint"] == int(g["vbm_kpoint"]) and p["cbm_kpoint"] == int(g["cbm_kpoint"]):
        assert p["is_direct_gap"] == bool(g["is_direct_gap"])
    assert p["nkpoints"] == int(g["nkpoints"]) and p["nbands"] == int(g["nbands"])
    mdg = float(g["minimum_direct_gap_eV"])
    if np.isnan(mdg):
        assert p["minimum_direct_gap_eV"] is None
    else:
        assert abs(p["minimum_direct_gap_eV"] - mdg) <= 1e-6
    if "dos2_grid" in g.files:
        r2 = E.Engine(ts).run(E.plan_batch([_struct(st, k, w)], ts), dos_range=(-20.0, 10.0), dos_points=1000,
                              dos_window=9.0)
        d2 = np.abs(r2.dos[0].cpu().numpy() - g["dos2_values"]).max()
        print(f"{case}: windowed 1000-point DOS err {d2:.2e}")
        assert d2 <= 1e-6


def test_drop_in_api_config0():
    g = golden("si_cfg0")
    st, tables, sd = load_case(g)
    model = M.MultiElementSkfParameterOptimizer.from_tables(tables)
    geom = M.Geometry(st["numbers"], st["positions"], st["cell"])
    props, ok = model.compute_multi_element_properties(geometry=geom, shell_dict=sd, kpoints=torch.tensor([8, 8, 8]),
                                                       get_fermi=True, device=DEV)
    assert ok is True
    for key in ("fermi_energy_eV", "fermi_energy_Ha", "band_gap_eV", "vbm_eV", "cbm_eV", "is_direct_gap",
                "vbm_kpoint", "cbm_kpoint", "valence_band_width_eV", "conduction_band_width_eV",
                "minimum_direct_gap_eV", "is_direct_semiconductor", "nkpoints", "nbands", "nelectrons",
                "dos_at_fermi", "dos_gap_center_eV", "dos_total_states", "dos_at_fermi_tensor",
                "dos_gap_center_tensor", "dos_total_states_tensor", "dos_energy_grid_tensor", "dos_values_tensor",
                "efermi", "bandgap", "calc", "eigenvalues"):
        assert key in props, key
    assert props["eigenvalues"].shape == (1, 512, 18)
    assert props["efermi"].shape == (1, 1, 1) and props["bandgap"].shape == (1,)
    assert np.abs(props["eigenvalues"][0].cpu().numpy() - g["eigenvalues"]).max() * H2E <= 1e-8
    assert abs(props["fermi_energy_eV"] - float(g["fermi_energy_eV"])) <= 1e-6
    assert props["nelectrons"] == int(g["nelectrons"])


def test_batch_is_invariant_to_composition():
    """Each structure's results are bitwise the same alone and inside a mixed batch (one table set)."""
    sts = syn.uneven_batch(6, nmin=2, nmax=20, zmax=30, seed=9, kdens=100.0)
    zs = sorted({int(z) for st in sts for z in st["numbers"]})
    sd = syn.default_shell_dict()
    ts = E.TableSet.from_synthetic(syn.make_tables(zs, sd, seed=9), {z: sd[z] for z in zs}, DEV)
    mixed = E.Engine(ts).run(E.plan_batch(sts, ts))
    same = lambda a, b: bool(((a == b) | (torch.isnan(a) & torch.isnan(b))).all())   # noqa: E731
    for s, st in enumerate(sts):
        alone = E.Engine(ts).run(E.plan_batch([st], ts))
        assert same(alone.eigenvalues(0), mixed.eigenvalues(s)), s
        assert same(alone.dos[0], mixed.dos[s]) and same(alone.stats[0], mixed.stats[s]), s


def test_random_structures_against_oracle():
    rng = np.random.default_rng(99)
    sts = []
    for n in (2, 3, 5, 8, 13):
        st = syn.random_structure(rng, n, zmax=65)
        st["kpoints"] = syn.gamma_centred_kpoints(syn.gamma_centred_grid(st["cell"], n, 40))
        sts.append(st)
    zs = sorted({int(z) for st in sts for z in st["numbers"]})
    sd = syn.default_shell_dict()
    tables = syn.make_tables(zs, sd, seed=7)
    ts = _tables(tables, sd)
    res = E.Engine(ts).run(E.plan_batch(sts, ts))
    worst = 0.0
    for s, st in enumerate(sts):
        H, S = O.hk_sk(st, tables, sd, st["kpoints"])
        try:
            e = O.eigh_generalized(H, S)
        except np.linalg.LinAlgError:
            assert (res.eig_status.cpu().numpy()[res.plan.prob_struct == s] != 0).any()
            continue
        worst = max(worst, np.abs(res.eigenvalues(s).cpu().numpy() - e).max() * H2E)
    print(f"random structures: worst eigenvalue error {worst:.2e} eV")
    assert worst <= 1e-8


def test_not_positive_definite_overlap_is_reported():
    """An overlap table far too large makes S(k) indefinite: status 2, NaN eigenvalues, no failure."""
    tables = syn.make_tables([14], {14: [0, 1]}, seed=0)
    for key in tables["pairs"][(14, 14)]["S"]:
        tables["pairs"][(14, 14)]["S"][key] = tables["pairs"][(14, 14)]["S"][key] * 40.0
    ts = _tables(tables, {14: [0, 1]})
    st = syn.diamond_si()
    st["kpoints"] = O.mp_kpoints([2, 2, 2])[0]
    res = E.Engine(ts).run(E.plan_batch([st], ts))
    stt = res.eig_status.cpu().numpy()
    H, S = O.hk_sk(st, tables, {14: [0, 1]}, st["kpoints"])
    spd = np.array([np.linalg.eigvalsh(S[q]).min() > 0 for q in range(len(S))])
    assert ((stt == 0) == spd).all()
    assert np.isnan(res.eigenvalues(0).cpu().numpy()[~spd]).all()
