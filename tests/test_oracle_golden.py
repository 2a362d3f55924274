"""Pin the CPU oracle to the reference's own outputs (golden fixtures)."""
import numpy as np
import pytest

from conftest import golden
from _cases import CASES, load_case, tables_checksum
from slakonet_gb300 import synthetic as syn
from oracle import slako_oracle as O

H2E = 27.211


def test_interp_bit_exact():
    g = golden("interp")
    out = O.interpolate(g["table"], float(g["step"]), g["r"])
    np.testing.assert_array_equal(out, g["values"])


@pytest.mark.parametrize("l1,l2", [(a, b) for a in range(4) for b in range(a, 4)])
def test_sk_blocks(l1, l2):
    g = golden("skblocks")
    out = O.sk_block(g["u"], l1, l2, g[f"ints_{l1}{l2}"])
    ref = g[f"block_{l1}{l2}"]
    assert np.abs(out - ref).max() <= 1e-13 * max(1.0, np.abs(ref).max())


def test_fermi_search():
    g = golden("fermi")
    n = len([k for k in g.files if k.startswith("eig_")])
    for c in range(n):
        eig = g[f"eig_{c}"]
        w = np.full(eig.shape[0], 1.0 / eig.shape[0])
        mu, it, conv = O.fermi_search(eig, w, float(g[f"ne_{c}"]))
        ref = float(g[f"mu_{c}"])
        if np.isnan(ref):
            assert np.isnan(mu) or not conv
        else:
            assert abs(mu - ref) * H2E <= 1e-6, (c, mu, ref)


@pytest.mark.parametrize("case", CASES)
def test_hk_sk_and_eigenvalues(case):
    g = golden(case)
    st, tables, sd = load_case(g)
    k = g["kpoints"]
    if "hk" in g.files:
        idx = g["hs_kindex"]
        H, S = O.hk_sk(st, tables, sd, k[idx])
        for M, R in ((H, g["hk"]), (S, g["sk"])):
            assert np.abs(M - R).max() <= 1e-12 * np.abs(R).max()
    # eigenvalues on a subset of k (all for small cases)
    sel = np.arange(len(k)) if len(k) <= 64 else np.linspace(0, len(k) - 1, 48).astype(int)
    H, S = O.hk_sk(st, tables, sd, k[sel])
    e = O.eigh_generalized(H, S)
    assert np.abs(e - g["eigenvalues"][sel]).max() * H2E <= 1e-8


@pytest.mark.parametrize("case", CASES)
def test_properties_from_reference_eigenvalues(case):
    g = golden(case)
    eig = g["eigenvalues"]
    w = g["k_weights"]
    p = O.properties(eig, w, float(g["nelectrons"]))
    assert abs(p["fermi_energy_eV"] - float(g["fermi_energy_eV"])) <= 1e-6
    assert abs(p["band_gap_eV"] - float(g["band_gap_eV"])) <= 1e-6
    assert abs(p["efermi"] - float(g["efermi_eV"])) <= 1e-6
    assert abs(p["bandgap"] - float(g["bandgap_eV"])) <= 1e-6
    np.testing.assert_array_equal(p["dos_energy_grid"], g["dos_energy_grid"])
    assert np.abs(p["dos_values"] - g["dos_values"]).max() <= 1e-6
    for key in ("vbm_eV", "cbm_eV", "valence_band_width_eV", "conduction_band_width_eV"):
        assert abs(p[key] - float(g[key])) <= 1e-6, key
    assert p["vbm_kpoint"] == int(g["vbm_kpoint"]) and p["cbm_kpoint"] == int(g["cbm_kpoint"])
    if "dos2_grid" in g.files:
        grid, dos = O.gaussian_dos(eig, w, O.fermi_search(eig, w, float(g["nelectrons"]))[0], (-20.0, 10.0), 1000, 0.1)
        np.testing.assert_array_equal(grid, g["dos2_grid"])
        assert np.abs(dos - g["dos2_values"]).max() <= 1e-6


def test_kpoint_generators():
    g = golden("si_cfg0")
    k, w = O.mp_kpoints([8, 8, 8])
    np.testing.assert_array_equal(k, g["kpoints"])
    g = golden("si_klines")
    k, w = O.klines_kpoints(g["klines"])
    assert np.abs(k - g["kpoints"]).max() <= 1e-15


@pytest.mark.parametrize("name", ["pdos_si", "pdos_gaas", "pdos_hfe"])
def test_oracle_atom_projected_dos_matches_reference(name):
    """The restatement on the reference's own eigenvectors reproduces its PDOS."""
    g = golden(name)
    from slakonet_gb300.elements import SYMBOLS
    types = [SYMBOLS[int(z)] for z in g["numbers"]]
    grid, pdos, unique = O.atom_projected_dos(g["eigenvalues"], g["eigenvectors"], types,
                                              float(g["fermi_energy_eV"]), 0.1, tuple(g["energy_range"]))
    assert unique == [str(u) for u in g["unique"]]
    np.testing.assert_array_equal(grid, g["grid"])
    err = max(np.abs(pdos[a] - g["pdos"][i]).max() for i, a in enumerate(unique))
    print(f"{name}: oracle PDOS vs reference {err:.1e}")
    assert err <= 1e-12


def test_oracle_atom_projected_dos_refuses_indivisible_orbitals():
    with pytest.raises(ValueError):
        O.atom_projected_dos(np.zeros((1, 5)), np.zeros((1, 5, 5)), ["H", "C"], 0.0)


def _ef_case(name):
    g = golden(name)
    zs = [int(z) for z in g["shell_z"]]
    full = syn.default_shell_dict()
    if name == "ef_si":
        sd = {14: [0, 1, 2]}
        tables = syn.make_tables(zs, sd, seed=int(g["table_seed"]))
    else:
        tables = syn.make_tables(zs, full, seed=int(g["table_seed"]))
        sd = {z: full[z] for z in zs}
    np.testing.assert_allclose(tables_checksum(tables), g["tables_checksum"], rtol=1e-12, atol=1e-300)
    st = {"numbers": g["numbers"], "positions": g["positions"], "cell": g["cell"]}
    return g, st, tables, sd


@pytest.mark.parametrize("name", ["ef_si", "ef_rand"])
def test_oracle_band_energy_matches_reference(name):
    g, st, tables, sd = _ef_case(name)
    e = O.band_energy(g["eigenvalues"], g["k_weights"], float(g["fermi_energy_Ha"]))
    print(f"{name}: band energy {e:.15f} vs reference {float(g['total_energy']):.15f}")
    assert abs(e - float(g["total_energy"])) <= 1e-12 * max(1.0, abs(e))


def test_oracle_finite_difference_forces_match_reference():
    g, st, tables, sd = _ef_case("ef_si")
    F = O.fd_forces(st, tables, sd)
    err = np.abs(F - g["forces"]).max()
    print(f"ef_si: oracle forces vs reference {err:.1e} (max |F| {np.abs(g['forces']).max():.3f})")
    assert err <= 1e-8
