"""Host-side logic and the C ABI library, without a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, golden
from oracle import slako_oracle as O
from slakonet_gb300 import _lib, engine as E, model as M, synthetic as syn


def header_functions():
    text = open(os.path.join(ROOT, "include", "slakonet_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^int\s+(skn_\w+)\s*\(", text, flags=re.M)))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = header_functions()
    assert len(names) >= 9
    for n in names:
        assert hasattr(lib, n), n
        assert n in _lib.SIGNATURES, n
    assert lib.skn_abi_version() == 100


def test_argument_errors_without_gpu():
    # invalid arguments are rejected before any launch
    assert _lib.load().skn_eigh_gen_batched(-1, None, None, None, None, None, None, None, None, None, 0, None) == 1
    assert _lib.load().skn_dos(1, None, None, None, None, None, None, None, 0.0, 1.0, 0, 0.1, 0.0,
                               None, None, None, None) == 1


def _walk_bonds(plan, s, cutoff):
    """numpy replica of the kernel's translation-box walk for structure s."""
    a0, a1 = plan.atom_ptr[s], plan.atom_ptr[s + 1]
    pos = plan.positions[a0:a1]
    cell = plan.cells[s]
    r = plan.image_range[s]
    T = np.array([[i, j, k] for i in range(-r[0], r[0] + 1) for j in range(-r[1], r[1] + 1)
                  for k in range(-r[2], r[2] + 1)], float)
    v = pos[None, None, :, :] + (T @ cell)[:, None, None, :] - pos[None, :, None, :]
    d = np.sqrt((v * v).sum(-1))
    c, i, j = np.nonzero((d < cutoff) & (d > 0))
    return set(zip(i.tolist(), j.tolist(), map(tuple, T[c].astype(int).tolist())))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_image_range_covers_every_bond(seed):
    rng = np.random.default_rng(seed)
    sts = []
    for n in (2, 5, 11):
        st = syn.random_structure(rng, n, zmax=30)
        st["kpoints"] = np.zeros((1, 3))
        sts.append(st)
    sts.append(dict(syn.diamond_si(), kpoints=np.zeros((1, 3))))
    zs = sorted({int(z) for st in sts for z in st["numbers"]})
    tables = syn.make_tables(zs, syn.default_shell_dict(), seed=seed)
    ts = E.TableSet.from_synthetic(tables, syn.default_shell_dict(), "cpu")
    plan = E.plan_batch(sts, ts)
    for s, st in enumerate(sts):
        i, j, T, d, u = O.bond_list(st["positions"], st["cell"], 10.0, rcut_images=30.0)
        ref = set(zip(i.tolist(), j.tolist(), map(tuple, T.tolist())))
        assert _walk_bonds(plan, s, 10.0) == ref


def test_plan_offsets_are_consistent():
    rng = np.random.default_rng(4)
    sts = []
    for n in (3, 7, 2):
        st = syn.random_structure(rng, n)
        st["kpoints"] = syn.gamma_centred_kpoints(syn.gamma_centred_grid(st["cell"], n, 50))
        sts.append(st)
    zs = sorted({int(z) for st in sts for z in st["numbers"]})
    ts = E.TableSet.from_synthetic(syn.make_tables(zs, syn.default_shell_dict(), seed=1), syn.default_shell_dict(), "cpu")
    p = E.plan_batch(sts, ts)
    assert p.hs_total == int(sum(int(p.nb[s]) ** 2 * int(p.nk[s]) for s in range(p.n_struct)))
    ends = p.hs_off + p.prob_n.astype(np.int64) ** 2
    assert ends.max() == p.hs_total and (p.hs_off[1:] == ends[:-1]).all()
    assert (p.eig_off_prob + p.prob_n <= p.eig_total).all()
    assert sorted(p.order.tolist()) == list(range(len(p.prob_n)))
    assert (np.diff(p.prob_n[p.order]) <= 0).all()
    nimg = np.prod(2 * p.image_range + 1, axis=1)
    assert p.n_phase == int((nimg * p.nk).sum())


def test_kpoint_generators_match_reference():
    g = golden("si_cfg0")
    np.testing.assert_array_equal(M.mp_kpoints([8, 8, 8]), g["kpoints"])
    g = golden("si_klines")
    assert np.abs(M.klines_kpoints(g["klines"]) - g["kpoints"]).max() <= 1e-15


def test_state_dict_layout_matches_reference_keys():
    tables = syn.make_tables([6, 14], syn.default_shell_dict(), seed=0)
    m = M.MultiElementSkfParameterOptimizer.from_tables(tables)
    keys = set(m.state_dict().keys())
    assert "skf_optimizers.Si-C.h_params.0-1" in keys
    assert "skf_optimizers.C-C.s_params.1-1" in keys
    p = m.skf_optimizers["Si-Si"].h_params["1-1"]
    assert p.dtype.is_floating_point and p.shape == (2, len(tables["grid"]))


def test_state_dict_round_trip_reloads_values_and_repacks_tables():
    import io
    import torch
    sd = {6: [0, 1], 14: [0, 1, 2]}
    src = M.MultiElementSkfParameterOptimizer.from_tables(syn.make_tables([6, 14], sd, seed=0))
    dst = M.MultiElementSkfParameterOptimizer.from_tables(syn.make_tables([6, 14], sd, seed=1))
    before = dst.table_set(sd, "cpu")
    buf = io.BytesIO()
    torch.save(src.state_dict(), buf)
    buf.seek(0)
    dst.load_state_dict(torch.load(buf))
    a, b = src.state_dict(), dst.state_dict()
    assert a.keys() == b.keys() and all(torch.equal(a[k], b[k]) for k in a)
    after = dst.table_set(sd, "cpu")                      # loading copies in place: the tables repack
    assert after is not before
    ref = src.table_set(sd, "cpu")
    assert torch.equal(after.tab_H, ref.tab_H) and torch.equal(after.tab_S, ref.tab_S)


def test_apply_constraints_clamps_to_band():
    tables = syn.make_tables([14], {14: [0, 1]}, seed=0)
    m = M.MultiElementSkfParameterOptimizer.from_tables(tables)
    p = m.skf_optimizers["Si-Si"].h_params["0-1"]
    o = p.detach().clone().numpy()
    with __import__("torch").no_grad():
        p.mul_(3.0)
    m.apply_constraints()
    lo = np.minimum(o * 0.7, o * 1.3)
    hi = np.maximum(o * 0.7, o * 1.3)
    v = p.detach().numpy()
    assert (v >= lo - 1e-15).all() and (v <= hi + 1e-15).all()


def test_engine_refuses_cpu():
    ts = E.TableSet.from_synthetic(syn.make_tables([1], {1: [0]}, seed=0), {1: [0]}, "cpu")
    with pytest.raises(_lib.SknError):
        E.Engine(ts)


def test_large_problem_routing_depends_on_each_problem_alone():
    n = np.array([18, 300, 1024, 1025, 2048, 2049, 4096, 4097, 9000])
    sizes = E.route_large(n)
    assert sizes.tolist() == [0, 0, 0, 4, 4, 8, 8, 12, 12]
    # the same problem gets the same path whatever else is in the batch
    for other in (np.array([5000] * 7), np.array([20] * 1000)):
        both = E.route_large(np.concatenate([n, other]))
        assert both[:len(n)].tolist() == sizes.tolist()
    # no threshold: only problems above the one-CTA bound move; a fixed cluster size overrides
    assert E.route_large(n, None).tolist() == [0, 0, 0, 0, 0, 8, 8, 12, 12]
    assert E.route_large(n, 0, 2).tolist() == [2] * len(n)


def test_real_kpoints_marked_in_plan():
    sd = syn.default_shell_dict()
    tables = syn.make_tables([14], sd, seed=0)
    ts = E.TableSet.from_synthetic(tables, {14: sd[14]}, "cpu")
    st = syn.diamond_si()
    st["kpoints"] = np.array([[0.0, 0.0, 0.0], [0.5, 0.0, -0.5], [0.25, 0.0, 0.0], [0.5, 1.0 / 3.0, 0.0]])
    plan = E.plan_batch([st], ts)
    assert plan.prob_real.tolist() == [True, True, False, False]


def test_device_tables_repack_exactly_when_parameters_change():
    sd = {6: [0, 1], 14: [0, 1, 2]}
    model = M.MultiElementSkfParameterOptimizer.from_tables(syn.make_tables([6, 14], sd, seed=1))
    ts = model.table_set(sd, "cpu")
    assert model.table_set(sd, "cpu") is ts                       # nothing changed: cached
    opt = model.skf_optimizers["C-Si"]
    key = next(iter(opt.h_params))
    import torch
    with torch.no_grad():
        opt.h_params[key].mul_(1.01)                               # in-place update (optimizer-style)
    ts2 = model.table_set(sd, "cpu")
    assert ts2 is not ts
    assert model.table_set(sd, "cpu") is ts2
    opt.apply_constraints()                                        # the reference's clamp, applied in place
    ts3 = model.table_set(sd, "cpu")
    assert ts3 is not ts2
    opt.h_params[key] = torch.nn.Parameter(opt.h_params[key].detach() * 1.0)   # entry replaced
    ts4 = model.table_set(sd, "cpu")
    assert ts4 is not ts3
    opt.h_params[key].data = opt.h_params[key].data * 2.0         # .data assignment is not tracked ...
    assert model.table_set(sd, "cpu") is ts4
    model.invalidate_tables()                                      # ... until invalidated
    assert model.table_set(sd, "cpu") is not ts4


def test_model_constraints_equal_the_per_pair_clamp():
    """The fused model-level clamp gives exactly the per-pair loop's values (including negative amplitudes)."""
    import copy
    import torch
    sd = {6: [0, 1], 14: [0, 1, 2]}
    a = M.MultiElementSkfParameterOptimizer.from_tables(syn.make_tables([6, 14], sd, seed=2))
    g = torch.Generator().manual_seed(0)
    with torch.no_grad():
        for p in a.parameters():
            p.mul_(1.0 + 0.4 * torch.randn(p.shape, generator=g, dtype=p.dtype))
    b = copy.deepcopy(a)
    a.apply_constraints()
    for opt in b.skf_optimizers.values():
        opt.apply_constraints()
    for (ka, pa), (kb, pb) in zip(a.named_parameters(), b.named_parameters()):
        assert ka == kb and torch.equal(pa, pb), ka
    a.apply_constraints()                      # idempotent
    for (ka, pa), (kb, pb) in zip(a.named_parameters(), b.named_parameters()):
        assert torch.equal(pa, pb), ka


def test_plan_batch_matches_per_structure_construction():
    """The whole-batch descriptor construction equals building each structure's arrays on its own."""
    sts = syn.uneven_batch(30, nmin=1, nmax=20, zmax=65, seed=21, kdens=200.0)
    sd = syn.default_shell_dict()
    zs = sorted({int(z) for st in sts for z in st["numbers"]})
    ts = E.TableSet.from_synthetic(syn.make_tables(zs, sd, seed=21), {z: sd[z] for z in zs}, "cpu")
    plan = E.plan_batch(sts, ts)
    a0 = o0 = 0
    for s, st in enumerate(sts):
        z = np.asarray(st["numbers"])
        sp = np.array([ts.sp_of[int(x)] for x in z])
        no = ts.sp_norb_np[sp]
        N = len(z)
        assert plan.atom_ptr[s] == a0 and plan.orb_ptr[s] == o0
        assert np.array_equal(plan.atom_species[a0:a0 + N], sp) and np.array_equal(plan.atom_norb[a0:a0 + N], no)
        assert np.array_equal(plan.atom_orb_off[a0:a0 + N], np.concatenate([[0], np.cumsum(no)[:-1]]))
        n = int(no.sum())
        assert np.array_equal(plan.orb_atom[o0:o0 + n], np.repeat(np.arange(N), no))
        assert np.array_equal(plan.onsite_H[o0:o0 + n], np.concatenate([ts.sp_onsite[q] for q in sp]))
        assert plan.nelec[s] == float(ts.sp_nelec[sp].sum())
        pb = int(plan.pair_base[s])
        assert np.array_equal(plan.pair_ni_nj[pb:pb + N * N], np.outer(no, no).reshape(-1))
        assert np.array_equal(plan.image_range[s], E.image_range(st["cell"], st["positions"], E.CUTOFF_BOHR))
        a0 += N
        o0 += n
    assert plan.atom_ptr[-1] == a0 and plan.orb_ptr[-1] == o0


def test_plan_rejects_malformed_structures_on_the_host():
    """Every flat offset the kernels use comes from these lengths, and the bond search loops over every
    lattice translation: malformed or degenerate input must stop in plan_batch, before any launch."""
    sd = {6: [0, 1], 14: [0, 1, 2]}
    ts = M.MultiElementSkfParameterOptimizer.from_tables(syn.make_tables([6, 14], sd, seed=0)).table_set(sd, "cpu")
    ok = {"numbers": np.array([6, 14]), "positions": np.array([[0.0, 0, 0], [1.5, 1.5, 1.5]]),
          "cell": np.eye(3) * 6.0, "kpoints": np.zeros((2, 3)), "weights": np.full(2, 0.5)}
    E.plan_batch([ok], ts)
    bad = {
        "no atoms": dict(ok, numbers=np.zeros(0, np.int64), positions=np.zeros((0, 3))),
        "positions for": dict(ok, positions=np.zeros((3, 3))),
        "no k-points": dict(ok, kpoints=np.zeros((0, 3)), weights=np.zeros(0)),
        "k-point weights": dict(ok, weights=np.ones(3)),
        "non-finite positions": dict(ok, positions=np.array([[0.0, 0, 0], [np.nan, 0, 0]])),
        "non-finite cell": dict(ok, cell=np.diag([6.0, np.inf, 6.0])),
        "non-finite kpoints": dict(ok, kpoints=np.array([[0.0, 0, 0], [np.inf, 0, 0]])),
        "singular cell": dict(ok, cell=np.array([[1.0, 0, 0], [2.0, 0, 0], [0, 0, 1.0]])),
        "too small or too flat": dict(ok, cell=np.array([[6.0, 0, 0], [0, 6.0, 0], [0, 0, 1e-4]])),
    }
    for msg, st in bad.items():
        with pytest.raises(ValueError, match=msg):
            E.plan_batch([ok, st], ts)
    with pytest.raises(ValueError, match="empty batch"):
        E.plan_batch([], ts)
    # the translation-times-pairs bound: 1000 atoms in a flat cell that alone would be allowed
    many = dict(ok, numbers=np.full(1000, 6), positions=np.random.default_rng(0).uniform(0, 6, (1000, 3)),
                cell=np.array([[6.0, 0, 0], [0, 6.0, 0], [0, 0, 0.005]]))
    with pytest.raises(ValueError, match="atom-pair translations"):
        E.plan_batch([many], ts)


def test_atom_projected_dos_rejects_mismatched_shapes_before_launch():
    import types
    import torch
    from slakonet_gb300 import compute_atom_projected_dos
    geom = M.Geometry([14, 14], np.zeros((2, 3)), np.eye(3) * 10)
    calc = types.SimpleNamespace(eigenvalue=torch.zeros(1, 3, 8),                     # nk 3, 8 bands
                                 eigenvectors=torch.zeros(1, 8, 8, 2, dtype=torch.complex128))   # nk 2
    with pytest.raises(ValueError, match="do not match"):
        compute_atom_projected_dos({"fermi_energy_eV": 0.0, "calc": calc}, geom)


def test_autotune_buckets_policies_and_cache_merge(tmp_path):
    from slakonet_gb300 import autotune as AT
    assert AT.buckets_up_to(492) == [16, 32, 64, 128, 256, 512]
    assert AT.buckets_up_to(16) == [16] and AT.buckets_up_to(5000) == AT.BUCKETS
    t = AT.Tuning({16: "_t64", 512: "_t256"})
    assert [t.shape_for(n) for n in (1, 16, 17, 300, 512, 513, 9000)] == ["_t64", "_t64", "", "_t256", "_t256", "", ""]
    pols = AT.candidate_policies(t)
    assert pols[0].choice == AT.Tuning.default().choice and len(pols) == 2
    assert all(set(p.choice) == set(AT.BUCKETS) for p in pols)
    assert not any(sh in ("_t32", "_t64") for p in pols for sh in p.choice.values())
    path = str(tmp_path / "cache" / "autotune.json")
    AT._merge_into_cache(path, "gpu-a", AT.Tuning({16: "_t64"}, {"16": {"_t64": 1.0}}))
    merged = AT._merge_into_cache(path, "gpu-a", AT.Tuning({512: "_t256"}, {"512": {"_t256": 2.0}}))
    assert merged.choice == {16: "_t64", 512: "_t256"} and set(merged.timings) == {"16", "512"}
    AT._merge_into_cache(path, "gpu-b", AT.Tuning({32: ""}))
    data = AT._read_cache(path)
    assert set(data) == {"gpu-a", "gpu-b"} and data["gpu-a"]["choice"] == {"16": "_t64", "512": "_t256"}
    assert not [f for f in os.listdir(os.path.dirname(path)) if f.endswith(".tmp")]


def test_index_range_guard_rejects_int32_overflow():
    n_at = np.array([2, 3])
    orb_cum = np.array([0, 4, 8, 13, 17, 21], dtype=np.int64)
    E._check_index_range(n_at, orb_cum, np.array([10, 20], np.int32), np.array([0, 8, 21], np.int64))
    with pytest.raises(ValueError, match="exceeds 2"):
        E._check_index_range(n_at, orb_cum, np.array([1, 300_000_000], np.int32), np.array([0, 8, 21], np.int64))
    with pytest.raises(ValueError, match="batch too large"):
        E._check_index_range(n_at, np.array([0, 2 ** 31], np.int64), np.array([1, 1], np.int32),
                             np.array([0, 1, 2], np.int64))


def test_eigensolver_groups_launch_few_long_problems_first():
    """The ~100 long real problems of the uneven batch go before the complex groups' full grids, and the many
    small problems last; the order depends on cost per problem in the group, not on the groups' input order."""
    n = np.array([492, 480, 300, 128, 100, 64, 40] * 10)
    real = np.zeros(len(n), bool)
    real[:2] = True                                                      # two long real problems
    idx = np.arange(len(n))
    big_real = idx[:2]
    big_complex = idx[(n >= 300) & ~real]
    small_complex = idx[(n < 300)]
    for groups in ([small_complex, big_complex, big_real], [big_complex, big_real, small_complex]):
        order = E.launch_order(groups, n, real)
        assert [groups[i] is big_real for i in order] == [True, False, False]
        assert groups[order[-1]] is small_complex
