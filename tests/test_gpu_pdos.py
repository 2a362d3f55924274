"""Atom-type projected DOS on the GPU against the reference's own output (needs a GB300).

The fixtures hold ``compute_atom_projected_dos`` (slakonet/predict_slakonet.py:119-210)
run by the reference on its eigenvectors.  Here the whole chain runs on the
GPU: H(k), S(k), eigenvectors, then the PDOS kernel.  Eigenvectors of
degenerate bands differ by a rotation inside their subspace, but the
per-type weights summed over the subspace, hence the PDOS, do not.
Gate: 1e-6 max abs (the DOS tolerance).
"""
import numpy as np
import pytest
import torch

from conftest import golden
from _cases import tables_checksum
from oracle import slako_oracle as O
from slakonet_gb300 import Geometry, compute_atom_projected_dos, model as M, synthetic as syn

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _case(name):
    g = golden(name)
    zs = [int(z) for z in g["shell_z"]]
    full = syn.default_shell_dict()
    if name == "pdos_si":
        sd = {14: [0, 1, 2]}
        tables = syn.make_tables(zs, sd, seed=int(g["table_seed"]))
    else:
        tables = syn.make_tables(zs, full, seed=int(g["table_seed"]))
        sd = {z: full[z] for z in zs}
    np.testing.assert_allclose(tables_checksum(tables), g["tables_checksum"], rtol=1e-12, atol=1e-300)
    return g, tables, sd


@pytest.mark.parametrize("name", ["pdos_si", "pdos_gaas", "pdos_hfe"])
def test_atom_projected_dos_matches_reference(name):
    g, tables, sd = _case(name)
    model = M.MultiElementSkfParameterOptimizer.from_tables(tables)
    geom = Geometry(g["numbers"], g["positions"], g["cell"])
    props, ok = model.compute_multi_element_properties(geometry=geom, shell_dict=sd,
                                                       kpoints=torch.tensor(g["mesh"]), get_fermi=True,
                                                       device=DEV, with_eigenvectors=True)
    assert abs(props["fermi_energy_eV"] - float(g["fermi_energy_eV"])) <= 1e-6
    grid, pdos, unique = compute_atom_projected_dos(props, props["calc"].geometry, sigma=0.1,
                                                    energy_range=tuple(g["energy_range"]))
    assert unique == [str(u) for u in g["unique"]]
    np.testing.assert_array_equal(grid, g["grid"])
    err = max(np.abs(pdos[a] - g["pdos"][i]).max() for i, a in enumerate(unique))
    print(f"{name}: GPU PDOS vs reference {err:.1e} (peak {g['pdos'].max():.2f})")
    assert err <= 1e-6


def test_pdos_kernel_on_reference_eigenvectors():
    """The kernel alone, fed the reference's eigenvectors, reproduces the reference to rounding."""
    g, tables, sd = _case("pdos_si")
    import types
    props = {"fermi_energy_eV": float(g["fermi_energy_eV"]),
             "calc": types.SimpleNamespace(eigenvalue=torch.as_tensor(g["eigenvalues"])[None],
                                           eigenvectors=torch.as_tensor(g["eigenvectors"]).permute(1, 2, 0)[None])}
    geom = Geometry(g["numbers"], g["positions"], g["cell"])
    grid, pdos, unique = compute_atom_projected_dos(props, geom, 0.1, tuple(g["energy_range"]))
    err = np.abs(pdos["Si"] - g["pdos"][0]).max()
    print(f"kernel on reference eigenvectors: {err:.1e}")
    assert err <= 1e-12


def test_indivisible_orbitals_raise_like_the_reference():
    import types
    props = {"fermi_energy_eV": 0.0,
             "calc": types.SimpleNamespace(eigenvalue=torch.zeros(1, 1, 5), eigenvectors=torch.zeros(1, 5, 5, 1,
                                                                                                   dtype=torch.complex128))}
    geom = Geometry([1, 6], np.zeros((2, 3)), np.eye(3) * 5)
    with pytest.raises(ValueError):
        compute_atom_projected_dos(props, geom)
