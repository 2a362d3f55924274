"""Checkpoints in the reference's ultra-compact format (slakonet/optim.py:485-625): a model written by
``save_ultra_compact`` reads back here, and -- where the reference package is installed beside the repository
(baseline/_ref) -- in the reference's own ``load_ultra_compact``, with every parameter bit for bit and each
pair's grid, cutoff and atomic data unchanged."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest
import torch

from conftest import ROOT
from slakonet_gb300 import model as M, synthetic as syn


def _fitted_model():
    zs = [6, 14]
    sd = syn.default_shell_dict()
    model = M.MultiElementSkfParameterOptimizer.from_tables(syn.make_tables(zs, {z: sd[z] for z in zs}, seed=5))
    g = torch.Generator().manual_seed(3)
    with torch.no_grad():               # stand-in for a fitting run: every parameter moved
        for p in model.parameters():
            p.mul_(1.0 + 0.01 * torch.randn(p.shape, generator=g, dtype=p.dtype))
    return model


def test_ultra_compact_round_trip(tmp_path):
    model = _fitted_model()
    path = model.save_ultra_compact(str(tmp_path / "fitted"))
    assert path.endswith("fitted.pt") and os.path.exists(path)
    torch.load(path, weights_only=True)               # tensors, numbers, strings, lists and dicts only
    back = M.MultiElementSkfParameterOptimizer.load_ultra_compact(path)
    a, b = model.state_dict(), back.state_dict()
    assert a.keys() == b.keys()
    assert all(torch.equal(a[k], b[k]) for k in a)
    for pk, opt in model.skf_optimizers.items():
        o2 = back.skf_optimizers[pk]
        assert o2.atom_pair == opt.atom_pair and o2.grid == opt.grid and o2.hs_cutoff == opt.hs_cutoff
        assert o2.atomic_data == opt.atomic_data


_REF_LOAD = r"""
import json, sys
sys.path.insert(0, sys.argv[1])
import refharness
ref = refharness.import_reference()
m = ref.optim.MultiElementSkfParameterOptimizer.load_ultra_compact(sys.argv[2])
sd = m.state_dict()
out = {k: [float(x) for x in v.reshape(-1)[:4]] + [float(v.double().sum()), list(v.shape)] for k, v in sd.items()}
meta = {k: {"atom_pair": list(o.atom_pair), "grid_len": len(o.grid), "hs_cutoff": float(o.hs_cutoff),
            "on_sites": (o.atomic_data or {}).get("on_sites")} for k, o in m.skf_optimizers.items()}
print(json.dumps({"params": out, "meta": meta}))
"""


def test_reference_reads_the_checkpoint(tmp_path):
    golden = os.path.join(ROOT, "tests", "golden")
    sys.path.insert(0, golden)
    try:
        import refharness
    finally:
        sys.path.remove(golden)
    if not os.path.isdir(os.path.join(refharness.REF_ROOT, "slakonet")):
        pytest.skip("the reference package is not installed beside the repository")
    model = _fitted_model()
    path = model.save_ultra_compact(str(tmp_path / "fitted.pt"))
    r = subprocess.run([sys.executable, "-c", _REF_LOAD, golden, path], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    got = json.loads(r.stdout.strip().splitlines()[-1])
    ours = model.state_dict()
    assert set(got["params"]) == set(ours)
    for k, v in ours.items():
        head = [float(x) for x in v.reshape(-1)[:4]]
        assert got["params"][k][:len(head)] == head, k
        assert got["params"][k][-2] == float(v.double().sum()) and got["params"][k][-1] == list(v.shape), k
    for pk, opt in model.skf_optimizers.items():
        m = got["meta"][pk]
        assert m["atom_pair"] == opt.atom_pair and m["grid_len"] == len(opt.grid) and m["hs_cutoff"] == opt.hs_cutoff
        assert m["on_sites"] == (opt.atomic_data or {}).get("on_sites")
    print(f"reference load_ultra_compact read {len(ours)} parameters of {len(model.skf_optimizers)} pairs")
