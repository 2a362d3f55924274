"""k-point reduction by time reversal (``model.reduce_time_reversal``), checked with the oracle: the reduced
list (about half the k-points, partner weights summed) gives every k-point's eigenvalues back through
``index`` and the same Fermi level, gap and DOS as the full list."""
import numpy as np
import pytest

from oracle import slako_oracle as O
from slakonet_gb300 import model as M, synthetic as syn

H2E = 27.211


@pytest.mark.parametrize("grid", ["gamma", "mp"])
def test_reduced_kpoints_give_the_full_lists_properties(grid):
    st = syn.uneven_batch(1, nmin=2, nmax=3, zmax=30, seed=11, kdens=300.0)[0]
    sd = syn.default_shell_dict()
    zs = sorted({int(z) for z in st["numbers"]})
    tables = syn.make_tables(zs, {z: sd[z] for z in zs}, seed=11)
    k = np.asarray(st["kpoints"]) if grid == "gamma" else M.mp_kpoints([4, 4, 3])
    w = np.full(len(k), 1.0 / len(k))
    k_red, w_red, index = M.reduce_time_reversal(k, w)
    assert len(k_red) <= 0.6 * len(k) and abs(w_red.sum() - 1.0) < 1e-14
    kw = dict(dos_range=(-20.0, 10.0), dos_points=1000)
    full = O.run_structure(st, tables, sd, k, w, **kw)
    red = O.run_structure(st, tables, sd, k_red, w_red, **kw)
    d_eig = np.abs(full["eigenvalues"] - red["eigenvalues"][index]).max() * H2E
    print(f"{grid}: {len(k)} -> {len(k_red)} k-points; eigenvalues {d_eig:.1e} eV")
    assert d_eig <= 1e-10
    assert np.abs(full["dos_values"] - red["dos_values"]).max() <= 1e-6
    if full["fermi_converged"] and red["fermi_converged"]:
        assert abs(full["fermi_energy_eV"] - red["fermi_energy_eV"]) <= 1e-6
        assert abs(full["band_gap_eV"] - red["band_gap_eV"]) <= 1e-6


def test_self_partnered_and_unpaired_points_keep_their_weight():
    k = np.array([[0.0, 0.0, 0.0], [0.5, 0.0, 0.0], [0.25, 0.0, 0.0], [0.75, 0.0, 0.0], [0.1, 0.2, 0.3]])
    w = np.array([0.1, 0.2, 0.3, 0.15, 0.25])
    k_red, w_red, index = M.reduce_time_reversal(k, w)
    assert len(k_red) == 4 and list(index) == [0, 1, 2, 2, 3]        # 0.75 = -0.25 + 1 pairs with 0.25
    assert np.allclose(w_red, [0.1, 0.2, 0.45, 0.25])
