"""Autotuned eigensolver launch shapes give the same eigenvalues as the default shape."""
import numpy as np
import pytest
import torch

from slakonet_gb300 import autotune as AT, engine as E, synthetic as syn

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def test_every_shape_and_the_tuned_dispatch_agree(tmp_path):
    rng = np.random.default_rng(8)
    sts = []
    for n in (1, 2, 4, 7, 12, 20):
        st = syn.random_structure(rng, n, zmax=65)
        st["kpoints"] = syn.gamma_centred_kpoints(syn.gamma_centred_grid(st["cell"], n, 60))
        sts.append(st)
    zs = sorted({int(z) for st in sts for z in st["numbers"]})
    sd = syn.default_shell_dict()
    ts = E.TableSet.from_synthetic(syn.make_tables(zs, sd, seed=5), sd, DEV)
    plan = E.plan_batch(sts, ts)
    ref = E.Engine(ts).run(plan).eig.clone()
    for sfx in AT.SHAPES:
        tun = AT.Tuning({u: sfx for u in AT.BUCKETS})
        out = E.Engine(ts, tuning=tun).run(plan).eig
        assert (out - ref).abs().max().item() * 27.211 <= 1e-10, sfx
    mixed = AT.Tuning({16: "_t64", 32: "_t64", 64: "", 128: "", 256: "_t256", 512: "_t256", 1024: "", 2048: ""})
    out = E.Engine(ts, tuning=mixed).run(plan).eig
    assert (out - ref).abs().max().item() * 27.211 <= 1e-10
    tun = AT.autotune(DEV, cache=str(tmp_path / "tune.json"), buckets=[16, 64, 256], budget_s=0.01)
    print("autotune choice:", tun.choice, tun.timings)
    assert set(tun.choice) == {16, 64, 256}
    again = AT.autotune(DEV, cache=str(tmp_path / "tune.json"), buckets=[16, 64, 256])
    assert again.choice == tun.choice
