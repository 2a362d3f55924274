"""A model read from DFTB+ .skf files runs the path exactly like the tables it was written from (needs a GB300)."""
import numpy as np
import pytest
import torch

from conftest import golden
from _cases import load_case
from slakonet_gb300 import model as M

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def test_skf_round_trip_gives_identical_results(tmp_path):
    g = golden("rand_a")
    st, tables, sd = load_case(g)
    a = M.MultiElementSkfParameterOptimizer.from_tables(tables)
    a.write_skf_files(str(tmp_path))
    b = M.MultiElementSkfParameterOptimizer.from_skf_files(str(tmp_path))
    s = dict(st, kpoints=g["kpoints"], weights=g["k_weights"])
    ra = a.compute_properties_batch([s], sd, DEV, dos_range=(-20.0, 10.0), dos_points=1000)
    rb = b.compute_properties_batch([s], sd, DEV, dos_range=(-20.0, 10.0), dos_points=1000)
    assert torch.equal(ra.eig, rb.eig) and torch.equal(ra.dos, rb.dos)
    de = np.abs(rb.eigenvalues(0).cpu().numpy() - g["eigenvalues"]).max() * 27.211
    print(f"rand_a through .skf files: eig error vs reference {de:.1e} eV")
    assert de <= 1e-8
