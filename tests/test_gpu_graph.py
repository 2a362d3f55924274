"""CUDA-graph replay of the path equals a fresh execution; refreshed tables are picked up."""
import numpy as np
import pytest
import torch

from slakonet_gb300 import engine as E, synthetic as syn

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _same(a, b):
    return bool(((a == b) | (torch.isnan(a) & torch.isnan(b))).all())


def test_graph_replay_matches_execute_and_tracks_table_updates():
    rng = np.random.default_rng(21)
    sts = []
    for n in (2, 5, 9, 3):
        st = syn.random_structure(rng, n, zmax=40)
        st["kpoints"] = syn.gamma_centred_kpoints(syn.gamma_centred_grid(st["cell"], n, 100))
        sts.append(st)
    zs = sorted({int(z) for st in sts for z in st["numbers"]})
    sd = syn.default_shell_dict()
    tables = syn.make_tables(zs, sd, seed=2)
    ts = E.TableSet.from_synthetic(tables, sd, DEV)
    eng = E.Engine(ts)
    plan = E.plan_batch(sts, ts)
    db = E.DeviceBatch(plan, DEV)
    kw = dict(dos_range=(-20.0, 10.0), dos_points=1000, dos_window=9.0)
    cap = E.CapturedPath(eng, db, **kw)
    ref = eng.execute(db, **kw)
    out = cap.replay()
    torch.cuda.synchronize()
    assert _same(out.eig, ref.eig) and _same(out.dos, ref.dos) and _same(out.stats, ref.stats)
    # new parameters: perturbed tables written into the captured buffers
    t2 = E.TableSet.from_synthetic(syn.perturb_tables(tables, 0.05, seed=3), sd, DEV)
    cap.refresh_tables(t2)
    out = cap.replay()
    ref2 = E.Engine(t2).execute(E.DeviceBatch(plan, DEV), **kw)
    torch.cuda.synchronize()
    assert _same(out.eig, ref2.eig) and _same(out.dos, ref2.dos)
    assert not _same(out.eig, ref.eig)
    print(f"graph: {cap.kernels_per_replay} kernels per replay")
