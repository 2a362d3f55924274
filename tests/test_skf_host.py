"""DFTB+ Slater-Koster file reading and writing (host only)."""
import os

import numpy as np
import pytest

from slakonet_gb300 import engine as E, model as M, skf as SKF, synthetic as syn


SAMPLE = """0.02, 4
-0.1 -0.2 -0.5 0.0 0.3 0.4 0.5 0.0 2.0 2.0
28.0855 8*0.0 1.0D0 10*0.0
1.0 2.0 3.0 4.0 5.0 6.0 7.0 8.0 9.0 10.0 10*0.5
2*1.5 8*0.0 0.25 0.125 0.0625 7*0.0
20*0.0
1.0D-1 2.0d-1 18*0.0
Spline
2 3.5
1.0 2.0 -0.5
2.0 3.0 0.1 0.2 0.3 0.4
3.0 3.5 0.1 0.2 0.3 0.4 0.5 0.6
"""


def test_read_simple_homonuclear_with_shorthand_commas_and_fortran_exponents():
    d = SKF.read_skf(SAMPLE, homonuclear=True)
    assert d["grid_step"] == 0.02 and d["n_grid"] == 4 and not d["extended"]
    a = d["atomic"]
    assert a["on_sites"] == [-0.5, -0.2, -0.1]            # s, p, d (file lists d first)
    assert a["hubbard_us"] == [0.5, 0.4, 0.3] and a["occupations"] == [2.0, 2.0, 0.0]
    assert a["mass"] == 28.0855 and d["r_poly"]["cutoff"] == 1.0
    H, S = d["H"], d["S"]
    # row 1: dd0..dd2 = 1,2,3  pd0,pd1 = 4,5  pp0,pp1 = 6,7  sd0 = 8  sp0 = 9  ss0 = 10
    assert H[(2, 2)][:, 0].tolist() == [1.0, 2.0, 3.0]
    assert H[(1, 2)][:, 0].tolist() == [4.0, 5.0] and H[(1, 1)][:, 0].tolist() == [6.0, 7.0]
    assert H[(0, 2)][0, 0] == 8.0 and H[(0, 1)][0, 0] == 9.0 and H[(0, 0)][0, 0] == 10.0
    assert S[(0, 0)][0, 0] == 0.5 and H[(2, 2)][:, 1].tolist() == [1.5, 1.5, 0.0]
    assert S[(0, 0)][0, 1] == 0.0 and S[(2, 2)][:, 1].tolist() == [0.25, 0.125, 0.0625]
    assert H[(2, 2)][0, 3] == 0.1 and H[(2, 2)][1, 3] == 0.2
    assert d["r_spline"]["cutoff"] == 3.5 and d["r_spline"]["exp_coef"] == [1.0, 2.0, -0.5]
    assert len(d["r_spline"]["segments"]) == 2 and len(d["r_spline"]["segments"][1]) == 8


def test_short_row_is_an_error():
    bad = "0.1 2\n" + "0 " * 20 + "\n" + "1.0 " * 20 + "\n" + "1.0 " * 19 + "\n"
    with pytest.raises(ValueError):
        SKF.read_skf(bad, homonuclear=False)


@pytest.mark.parametrize("shells", [{6: [0, 1], 14: [0, 1, 2]}, {60: [0, 1, 2, 3], 1: [0]}])
def test_write_read_round_trip_is_exact(tmp_path, shells):
    tables = syn.make_tables(list(shells), shells, seed=3)
    for (za, zb), pair in tables["pairs"].items():
        atomic = None
        if za == zb:
            el = tables["elements"][za]
            atomic = {"on_sites": list(el["on_sites"]), "occupations": list(el["occupations"]), "mass": 12.5}
        path = os.path.join(tmp_path, f"{za}-{zb}.skf")
        SKF.write_skf(path, pair["H"], pair["S"], tables["step"], atomic)
        d = SKF.read_skf(path, homonuclear=(za == zb))
        assert d["grid_step"] == tables["step"] and d["n_grid"] == len(tables["grid"])
        for key in pair["H"]:
            assert np.array_equal(d["H"][key], pair["H"][key]) and np.array_equal(d["S"][key], pair["S"][key])
        if atomic:
            n = len(atomic["on_sites"])
            assert d["atomic"]["on_sites"][:n] == atomic["on_sites"]


def test_model_from_skf_directory_matches_tables(tmp_path):
    sd = {6: [0, 1], 14: [0, 1, 2]}
    tables = syn.make_tables([6, 14], sd, seed=5)
    ref = M.MultiElementSkfParameterOptimizer.from_tables(tables)
    ref.write_skf_files(str(tmp_path))
    assert sorted(os.listdir(tmp_path)) == ["C-C.skf", "C-Si.skf", "Si-C.skf", "Si-Si.skf"]
    got = M.MultiElementSkfParameterOptimizer.from_skf_files(str(tmp_path))
    assert set(got.skf_optimizers) == set(ref.skf_optimizers)
    for key, opt in ref.skf_optimizers.items():
        g = got.skf_optimizers[key]
        assert g.grid == opt.grid and g.atom_pair == opt.atom_pair
        for k, v in opt.h_params.items():
            assert np.array_equal(g.h_params[k].detach().numpy(), v.detach().numpy())
        for k, v in opt.s_params.items():
            assert np.array_equal(g.s_params[k].detach().numpy(), v.detach().numpy())
    ts_a = ref.table_set(sd, "cpu")
    ts_b = got.table_set(sd, "cpu")
    assert np.array_equal(ts_a.sp_nelec, ts_b.sp_nelec)
