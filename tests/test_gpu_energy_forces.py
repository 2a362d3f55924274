"""get_energy and get_forces through the drop-in API against the reference (needs a GB300).

Fixtures: the reference's compute_multi_element_properties(get_energy=True,
get_forces=True): Fermi-smeared band energy (slakonet/main.py:1430-1448) and
central-difference forces on the eigenvalue sum at a 5x5x5 grid
(slakonet/main.py:198-281).  Here the band energy comes out of the Fermi
kernel and the 6N displaced structures run as one batch.
Gates: band energy 1e-10 Hartree, forces 1e-8 Hartree/Bohr.
"""
import numpy as np
import pytest
import torch

from conftest import golden
from _cases import tables_checksum
from slakonet_gb300 import Geometry, model as M, synthetic as syn

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


@pytest.mark.parametrize("name", ["ef_si", "ef_rand"])
def test_energy_and_forces_match_reference(name):
    g = golden(name)
    zs = [int(z) for z in g["shell_z"]]
    full = syn.default_shell_dict()
    sd = {14: [0, 1, 2]} if name == "ef_si" else {z: full[z] for z in zs}
    tables = syn.make_tables(zs, sd if name == "ef_si" else full, seed=int(g["table_seed"]))
    np.testing.assert_allclose(tables_checksum(tables), g["tables_checksum"], rtol=1e-12, atol=1e-300)
    model = M.MultiElementSkfParameterOptimizer.from_tables(tables)
    geom = Geometry(g["numbers"], g["positions"], g["cell"])
    props, ok = model.compute_multi_element_properties(geometry=geom, shell_dict=sd, kpoints=torch.tensor(g["mesh"]),
                                                       get_fermi=True, get_energy=True, get_forces=True, device=DEV)
    de = abs(float(props["total_energy"]) - float(g["total_energy"]))
    F = props["forces"][0].cpu().numpy()
    dF = np.abs(F - g["forces"]).max()
    print(f"{name}: band energy err {de:.1e} Ha, forces err {dF:.1e} Ha/Bohr (max |F| {np.abs(g['forces']).max():.3f})")
    assert props["forces"].shape == (1, len(g["numbers"]), 3)
    assert de <= 1e-10 and dF <= 1e-8
