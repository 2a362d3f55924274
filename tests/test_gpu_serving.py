"""Continuous-batching server on the GPU: results alone equal results in the mix.

The mix includes two structures of more than 1024 orbitals, whose k-points run
on the cluster eigensolver, so both eigensolver paths are covered."""
import numpy as np
import pytest
import torch

from slakonet_gb300 import engine as E, model as M, serving as SV, synthetic as syn

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def test_results_identical_alone_and_in_the_mix():
    rng = np.random.default_rng(11)
    sts = []
    for i in range(40):
        n = int(round(np.exp(rng.uniform(0, np.log(30)))))
        st = syn.random_structure(rng, max(n, 1), zmax=65)
        st["kpoints"] = syn.gamma_centred_kpoints(syn.gamma_centred_grid(st["cell"], len(st["numbers"]), 200))
        st["weights"] = np.full(len(st["kpoints"]), 1.0 / len(st["kpoints"]))
        sts.append(st)
    for pos, n_atoms in ((7, 130), (23, 140)):      # 9 orbitals per atom (Z = 21..30): n > 1024
        st = syn.random_structure(rng, n_atoms, zmax=30)
        st["numbers"] = 21 + (np.asarray(st["numbers"]) % 10)
        st["kpoints"] = syn.gamma_centred_kpoints((1, 1, 2))
        st["weights"] = np.full(2, 0.5)
        sts.insert(pos, st)
    zs = sorted({int(z) for st in sts for z in st["numbers"]})
    sd = syn.default_shell_dict()
    # the server sends problems above 512 orbitals to the cluster eigensolver, compute_properties_batch those
    # above 1024: no structure here falls between, so both run every problem on the same kernel
    norb = [sum(sum(2 * l + 1 for l in sd[int(z)]) for z in st["numbers"]) for st in sts]
    assert not any(512 < n <= 1024 for n in norb)
    tables = syn.make_tables(zs, sd, seed=4)
    model = M.MultiElementSkfParameterOptimizer.from_tables(tables)
    server = SV.Server(model, sd, DEV, species=zs, n_workers=3, mem_budget_bytes=1 << 30)
    lat, wall, res = SV.poisson_stream(server, sts, rate=400.0, seed=2)
    server.close()
    errs = [r["error"] for r in res if "error" in r]
    assert not errs, errs[:3]
    assert len(lat) == len(sts) and server.batches >= 2
    print(f"served {len(sts)} structures in {server.batches} batches: p50 {1e3*np.percentile(lat, 50):.1f} ms, "
          f"p99 {1e3*np.percentile(lat, 99):.1f} ms")
    for st, r in zip(sts, res):
        alone = model.compute_properties_batch([st], sd, DEV, dos_range=(-20.0, 10.0), dos_points=1000,
                                               dos_window=9.0)
        same = lambda a, b: bool(((a == b) | (torch.isnan(a) & torch.isnan(b))).all())
        assert same(alone.eigenvalues(0).cpu(), r["eigenvalues"])
        assert same(alone.dos[0].cpu(), r["dos"])
        assert same(alone.stats[0].cpu(), r["stats"])
