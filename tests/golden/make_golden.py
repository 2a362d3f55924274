"""Generate the golden fixtures by running the reference SlakoNet code.

Run in a container that has the reference source, with ``SLAKONET_REF`` naming the
directory that holds its ``slakonet`` package:

    SLAKONET_REF=<reference checkout> python tests/golden/make_golden.py

Every fixture is produced by the reference's own functions on seeded
synthetic inputs from ``slakonet_gb300.synthetic``; the numbers are frozen
as ``.npz`` files beside this script.  Tests compare the CPU oracle and the
CUDA path against them; nothing at test time needs the reference.
"""
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

from refharness import import_reference, build_reference_model  # noqa: E402
from slakonet_gb300 import synthetic as syn  # noqa: E402

ref = import_reference()
torch.set_default_dtype(torch.float64)


def tables_checksum(tables):
    acc = []
    for pk in sorted(tables["pairs"]):
        for kind in ("H", "S"):
            for key in sorted(tables["pairs"][pk][kind]):
                t = tables["pairs"][pk][kind][key]
                acc.append([np.abs(t).sum(), t[:, 100].sum(), t[:, -1].sum()])
    for z in sorted(tables["elements"]):
        acc.append([np.sum(tables["elements"][z]["on_sites"]), np.sum(tables["elements"][z]["occupations"]), 0.0])
    return np.array(acc)


def geometry(st):
    return ref.atoms.Geometry(torch.tensor(st["numbers"]).unsqueeze(0),
                              torch.tensor(st["positions"]).unsqueeze(0),
                              cell=torch.tensor(st["cell"]).unsqueeze(0))


class inject_kpoints:
    """Replace ``Periodic._kpoints`` (slakonet/atoms.py:359-392) with a fixed list.

    The reference's public API only builds offset Monkhorst-Pack grids or
    k-lines; Gamma-centred grids are injected here.
    """

    def __init__(self, k):
        self.k = torch.tensor(np.asarray(k, dtype=np.float64))

    def __enter__(self):
        P = ref.atoms.Periodic
        self.orig = P._kpoints
        k = self.k

        def _kp(this, **kwargs):
            nk = len(k)
            return k.unsqueeze(0), torch.tensor([nk]), torch.full((1, nk), 1.0 / nk)
        P._kpoints = _kp
        return self

    def __exit__(self, *a):
        ref.atoms.Periodic._kpoints = self.orig


def run_reference(model, st, shell_dict, kpoints=None, mesh=None, klines=None, keep_hs=None,
                  extra_dos=None):
    geom = geometry(st)
    kw = dict(geometry=geom, shell_dict=shell_dict, device="cpu", get_fermi=True)
    ctx = inject_kpoints(kpoints) if kpoints is not None else None
    if mesh is not None:
        kw["kpoints"] = torch.tensor(mesh)
    if klines is not None:
        kw["klines"] = torch.tensor(klines)
    with torch.no_grad():
        if ctx:
            with ctx:
                props, ok = model.compute_multi_element_properties(**kw)
        else:
            props, ok = model.compute_multi_element_properties(**kw)
    calc = props["calc"]
    out = {
        "eigenvalues": props["eigenvalues"][0].numpy(),
        "kpoints": calc.kpoints[0].numpy(),
        "k_weights": calc.k_weights[0].numpy(),
        "dos_energy_grid": props["dos_energy_grid_tensor"].numpy(),
        "dos_values": props["dos_values_tensor"].numpy(),
        "efermi_eV": props["efermi"].reshape(-1)[0].item(),
        "bandgap_eV": props["bandgap"].reshape(-1)[0].item(),
        "nelectrons": calc.nelectron.item(),
    }
    for key in ("fermi_energy_eV", "fermi_energy_Ha", "vbm_eV", "cbm_eV", "vbm_kpoint", "cbm_kpoint",
                "valence_band_width_eV", "conduction_band_width_eV", "dos_at_fermi", "dos_gap_center_eV",
                "dos_total_states", "nkpoints", "nbands"):
        out[key] = np.float64(props[key])
    out["band_gap_eV"] = float(props["band_gap_eV"])
    out["is_direct_gap"] = bool(props["is_direct_gap"])
    mdg = props["minimum_direct_gap_eV"]
    out["minimum_direct_gap_eV"] = np.nan if mdg is None else float(mdg)
    out["is_direct_semiconductor"] = bool(props["is_direct_semiconductor"])
    if keep_hs is not None:
        out["hk"] = calc.ham[0].permute(2, 0, 1)[keep_hs].numpy()
        out["sk"] = calc.overlap[0].permute(2, 0, 1)[keep_hs].numpy()
        out["hs_kindex"] = np.asarray(keep_hs)
    if extra_dos is not None:
        lo, hi, npts = extra_dos
        with torch.no_grad():
            g, d = calc.calculate_dos(energy_range=(lo, hi), num_points=npts, sigma=0.1)
        out["dos2_grid"] = g.numpy()
        out["dos2_values"] = d.numpy()
    return out


def fixture_pdos(name, st, shell_dict, table_seed, mesh, energy_range=(-10.0, 10.0)):
    """Atom-type projected DOS from the reference's own ``compute_atom_projected_dos``
    (slakonet/predict_slakonet.py:119-210) on its eigenvectors (with_eigenvectors=True)."""
    zs = sorted({int(z) for z in st["numbers"]})
    tables = syn.make_tables(zs, syn.default_shell_dict() if shell_dict is None else shell_dict, seed=table_seed)
    sd = {z: (shell_dict or syn.default_shell_dict())[z] for z in zs}
    model = build_reference_model(ref, tables)
    geom = geometry(st)
    with torch.no_grad():
        props, ok = model.compute_multi_element_properties(geometry=geom, shell_dict=sd, kpoints=torch.tensor(mesh),
                                                           device="cpu", get_fermi=True, with_eigenvectors=True)
        grid, pdos, unique = ref.predict.compute_atom_projected_dos(props, geom, sigma=0.1,
                                                                    energy_range=energy_range)
    calc = props["calc"]
    payload = dict(numbers=st["numbers"], positions=st["positions"], cell=st["cell"], mesh=np.array(mesh),
                   table_seed=table_seed, tables_checksum=tables_checksum(tables),
                   shells=np.array([len(sd[z]) for z in zs]), shell_z=np.array(zs),
                   energy_range=np.array(energy_range), fermi_energy_eV=float(props["fermi_energy_eV"]),
                   eigenvalues=calc.eigenvalue[0].numpy(),
                   eigenvectors=calc.eigenvectors[0].permute(2, 0, 1).numpy(),   # [nk, component, band]
                   grid=grid, unique=np.array(unique),
                   pdos=np.stack([pdos[a] for a in unique]))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **payload)
    print(name, "pdos", {a: float(np.trapezoid(pdos[a], grid)) for a in unique})


def fixture_interp():
    rng = np.random.default_rng(11)
    grid = syn.grid_points()
    tab = rng.standard_normal((4, len(grid))).cumsum(1) * 0.01 * np.exp(-0.3 * grid)[None]
    r = np.concatenate([rng.uniform(1e-3, 14.0, 400), [0.02, 0.1, 0.179, 13.2, 13.22, 13.24, 13.5, 14.0, 14.2, 14.23]])
    pi = ref.interp.PolyInterpU(torch.tensor(grid), torch.tensor(tab.T))
    vals = pi(torch.tensor(r)).numpy()
    np.savez_compressed(os.path.join(HERE, "interp.npz"), table=tab, step=0.02, r=r, values=vals)


def fixture_blocks():
    rng = np.random.default_rng(12)
    u = rng.standard_normal((64, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    # include axis-aligned and near-axis directions
    u[:6] = [[0, 0, 1], [0, 0, -1], [1, 0, 0], [0, 1, 0], [0, -1, 0], [-1, 0, 0]]
    u[6] = np.array([1e-9, 2e-9, 1.0]) / np.linalg.norm([1e-9, 2e-9, 1.0])
    out = {"u": u}
    for l1 in range(4):
        for l2 in range(l1, 4):
            ints = rng.standard_normal((64, l1 + 1))
            blk = ref.sk.sub_block_rot(torch.tensor([l1, l2]), torch.tensor(u), torch.tensor(ints)).numpy()
            out[f"ints_{l1}{l2}"] = ints
            out[f"block_{l1}{l2}"] = blk
    np.savez_compressed(os.path.join(HERE, "skblocks.npz"), **out)


def save_case(name, tables, data, extra):
    payload = dict(data)
    payload.update(extra)
    payload["tables_checksum"] = tables_checksum(tables)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **payload)


def fixture_si_cfg0():
    sd = {14: [0, 1, 2]}
    tables = syn.make_tables([14], sd, seed=0)
    model = build_reference_model(ref, tables)
    st = syn.diamond_si()
    data = run_reference(model, st, sd, mesh=[8, 8, 8], keep_hs=[0, 1, 77, 300, 511],
                         extra_dos=(-20.0, 10.0, 1000))
    save_case("si_cfg0", tables, data, {"numbers": st["numbers"], "positions": st["positions"],
                                         "cell": st["cell"], "seed": 0, "shells": np.array([0, 1, 2])})


def fixture_random(name, n_atoms, struct_seed, table_seed, zmax=65, mesh=None, numbers=None):
    rng = np.random.default_rng(struct_seed)
    st = syn.random_structure(rng, n_atoms, zmax=zmax)
    if numbers is not None:
        st["numbers"] = np.array(numbers)
    sd_all = syn.default_shell_dict()
    sd = {int(z): sd_all[int(z)] for z in st["numbers"]}
    tables = syn.make_tables(st["numbers"], sd_all, seed=table_seed)
    model = build_reference_model(ref, tables)
    if mesh is None:
        mesh = syn.gamma_centred_grid(st["cell"], n_atoms)
    k = syn.gamma_centred_kpoints(mesh)
    keep = sorted(set([0, len(k) // 2, len(k) - 1]))
    data = run_reference(model, st, sd, kpoints=k, keep_hs=keep, extra_dos=(-20.0, 10.0, 1000))
    save_case(name, tables, data, {"numbers": st["numbers"], "positions": st["positions"],
                                    "cell": st["cell"], "mesh": np.array(mesh), "table_seed": table_seed})


def fixture_klines():
    sd = {14: [0, 1, 2]}
    tables = syn.make_tables([14], sd, seed=0)
    model = build_reference_model(ref, tables)
    st = syn.diamond_si()
    kl = np.array([[0.0, 0.0, 0.0, 0.5, 0.5, 0.0, 12],
                   [0.5, 0.5, 0.0, 0.5, 0.25, 0.75, 7],
                   [0.5, 0.25, 0.75, 0.0, 0.0, 0.0, 9]])
    data = run_reference(model, st, sd, klines=kl)
    save_case("si_klines", tables, data, {"numbers": st["numbers"], "positions": st["positions"],
                                           "cell": st["cell"], "klines": kl, "seed": 0,
                                           "shells": np.array([0, 1, 2])})


def fixture_fermi():
    """Reference ``fermi_search`` on assorted eigenvalue sets, including divergent ones."""
    rng = np.random.default_rng(13)
    cases = {}
    for c in range(12):
        nk, nb = int(rng.integers(1, 40)), int(rng.integers(2, 30))
        eig = np.sort(rng.normal(-0.2, 0.3, (nk, nb)), axis=1)
        if c % 3 == 1:
            eig[:, nb // 2:] += 0.2   # gapped
        w = np.full(nk, 1.0 / nk)
        ne = float(rng.integers(1, 2 * nb))
        mu = ref.fermi.fermi_search(torch.tensor(eig)[None], torch.tensor([ne]), torch.tensor(w)[None]).detach()
        cases[f"eig_{c}"] = eig
        cases[f"ne_{c}"] = np.float64(ne)
        cases[f"mu_{c}"] = mu.reshape(-1)[0].item()
    np.savez_compressed(os.path.join(HERE, "fermi.npz"), **cases)


def _fixed_symeig_backward(ctx, w_bar, v_bar):
    """_SymEigB.backward (slakonet/utils.py:387-473) with the eigenvector conjugate restored."""
    w, v = ctx.saved_tensors
    bf = ctx.bf
    vh = v.conj().transpose(-2, -1)
    out = v @ torch.diag_embed(w_bar.to(v.dtype)) @ vh
    if v_bar is not None:
        d = w.unsqueeze(-2) - w.unsqueeze(-1)
        d = torch.where(d.abs() > bf, d, torch.full_like(d, bf) * torch.sign(d))
        Fm = torch.where(torch.eye(w.shape[-1], dtype=torch.bool), torch.zeros_like(d), 1.0 / d)
        x = Fm.to(v.dtype) * (vh @ v_bar)
        out = out + v @ ((x + x.conj().transpose(-2, -1)) / 2) @ vh
    return out, None, None


def _reference_grads(model, st, sd, kpoints, fixed):
    """Gradients of L = sum sin(5 e + 0.3) over all (k, band) eigenvalues (Hartree)."""
    orig = ref.utils._SymEigB.backward
    if fixed:
        ref.utils._SymEigB.backward = staticmethod(_fixed_symeig_backward)
    try:
        model.zero_grad()
        with inject_kpoints(kpoints):
            props, _ = model.compute_multi_element_properties(geometry=geometry(st), shell_dict=sd, device="cpu")
        eig = props["eigenvalues"]
        loss = torch.sin(5.0 * eig + 0.3).sum()
        loss.backward()
    finally:
        ref.utils._SymEigB.backward = orig
    out = {}
    for key, opt in model.skf_optimizers.items():
        for kind, pd in (("h", opt.h_params), ("s", opt.s_params)):
            for lk, prm in pd.items():
                out[f"{key}|{kind}|{lk}"] = (prm.grad.detach().numpy().copy() if prm.grad is not None
                                             else np.zeros(tuple(prm.shape)))
    return out, float(loss.detach())


def _reference_loss(model, st, sd, kpoints):
    with torch.no_grad(), inject_kpoints(kpoints):
        props, _ = model.compute_multi_element_properties(geometry=geometry(st), shell_dict=sd, device="cpu")
    return float(torch.sin(5.0 * props["eigenvalues"] + 0.3).sum())


def fixture_gradients():
    """Reference autograd (shipped and conjugate-restored) plus central differences, h = 1e-5."""
    cases = []
    sd = {14: [0, 1, 2]}
    tables = syn.make_tables([14], sd, seed=0)
    cases.append(("grad_si", tables, syn.diamond_si(), sd, np.array([[0.1, 0.2, 0.3], [0.0, 0.0, 0.0],
                                                                    [0.25, 0.5, 0.125]]), {"seed": 0,
                                                                                           "shells": np.array([0, 1, 2])}))
    rng = np.random.default_rng(31)
    st = syn.random_structure(rng, 3, zmax=30)
    st["numbers"] = np.array([1, 26, 14])
    sd_all = syn.default_shell_dict()
    tables2 = syn.make_tables(st["numbers"], sd_all, seed=9)
    cases.append(("grad_hetero", tables2, st, {int(z): sd_all[int(z)] for z in st["numbers"]},
                  np.array([[0.0, 0.0, 0.0], [0.3, -0.2, 0.1]]), {"table_seed": 9}))
    for name, tb, stx, sdx, kp, extra in cases:
        model = build_reference_model(ref, tb)
        g_ship, loss = _reference_grads(model, stx, sdx, kp, fixed=False)
        g_fix, _ = _reference_grads(model, stx, sdx, kp, fixed=True)
        # central differences on the entries with the largest fixed gradients
        keys = sorted(g_fix, key=lambda k: -np.abs(g_fix[k]).max())[:3]
        fd = []
        for key in keys:
            pair, kind, lk = key.split("|")
            prm = getattr(model.skf_optimizers[pair], f"{kind}_params")[lk]
            idx = np.unravel_index(np.argmax(np.abs(g_fix[key])), g_fix[key].shape)
            with torch.no_grad():
                old = prm[idx].item()
                prm[idx] = old + 1e-5
                lp = _reference_loss(model, stx, sdx, kp)
                prm[idx] = old - 1e-5
                lm = _reference_loss(model, stx, sdx, kp)
                prm[idx] = old
            fd.append((key, idx, (lp - lm) / 2e-5, g_fix[key][idx], g_ship[key][idx]))
        payload = {"kpoints": kp, "numbers": stx["numbers"], "positions": stx["positions"], "cell": stx["cell"],
                   "loss": loss, "tables_checksum": tables_checksum(tb)}
        payload.update(extra)
        for k, v in g_fix.items():
            payload["fixed|" + k] = v
            payload["shipped|" + k] = g_ship[k]
        payload["fd_keys"] = np.array([f[0] for f in fd])
        payload["fd_idx"] = np.array([list(f[1]) for f in fd])
        payload["fd_values"] = np.array([[f[2], f[3], f[4]] for f in fd])
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **payload)
        print(name, "FD | fixed autograd | shipped autograd:")
        for f in fd:
            print("  ", f[0], f[1], f"{f[2]: .6e} {f[3]: .6e} {f[4]: .6e}")


TRAIN_LR = 1e-3
TRAIN_STEPS = 3


def _train_structures(seed):
    """Two small C/Si cells with Gamma-centred 3x3x2 grids (complex k-points among them)."""
    rng = np.random.default_rng(seed)
    out = []
    for numbers in ([6, 14, 14], [14, 6, 6, 14]):
        st = syn.random_structure(rng, len(numbers), zmax=14)
        st["numbers"] = np.array(numbers)
        st["kpoints"] = syn.gamma_centred_kpoints((3, 3, 2))
        out.append(st)
    return out


def _train_forward(model, st, sd):
    """The reference's properties call with gradients, then the 1000-point DOS on [-20, 10] eV of the
    fitting workload from its own calculate_dos (slakonet/main.py:709-797)."""
    try:
        with inject_kpoints(st["kpoints"]):
            props, ok = model.compute_multi_element_properties(geometry=geometry(st), shell_dict=sd, device="cpu",
                                                               get_fermi=True)
    except IndexError:          # every k-point dropped: the reference packs an empty list
        raise ValueError("the reference dropped every k-point (S(k) not positive definite)")
    if props["eigenvalues"].shape[1] != len(st["kpoints"]):
        raise ValueError("the reference dropped k-points whose S(k) is not positive definite")
    _, dos = props["calc"].calculate_dos(energy_range=(-20.0, 10.0), num_points=1000, sigma=0.1)
    return dos, props["band_gap_eV"]


def fixture_training():
    """The first structure seed (from 77) whose two cells keep every S(k) positive definite over the three
    steps (apply_constraints rescales negative and small overlap entries, which can break definiteness)."""
    for seed in range(77, 120):
        try:
            return _fixture_training(seed)
        except ValueError as e:
            print(f"structure seed {seed}: {e}")
    raise RuntimeError("no structure seed kept S(k) positive definite")


def _fixture_training(struct_seed):
    """Three steps of the reference's fitting loop (slakonet/optim.py:1656-1772) on two structures:
    apply_constraints, per-structure loss weighted by atom count, 1e-10 * sum(theta^2), backward with the
    eigenvector conjugate restored in _SymEigB.backward, gradient clipping at 2.0, AdamW, ReduceLROnPlateau.
    The per-structure loss is the fitting workload's DOS MSE plus band-gap absolute error, against targets
    from the same reference call on tables with 5 % perturbed amplitudes (seed 1)."""
    sd_all = syn.default_shell_dict()
    sd = {6: sd_all[6], 14: sd_all[14]}
    tables = syn.make_tables([6, 14], sd, seed=4)
    sts = _train_structures(struct_seed)
    target_model = build_reference_model(ref, syn.perturb_tables(tables, 0.05, 1))
    dos_t, gap_t = [], []
    with torch.no_grad():
        for st in sts:
            d, g = _train_forward(target_model, st, sd)
            dos_t.append(d.clone())
            gap_t.append(float(g))
    model = build_reference_model(ref, tables)
    opt = torch.optim.AdamW(model.parameters(), lr=TRAIN_LR)
    sched = torch.optim.lr_scheduler.ReduceLROnPlateau(opt, mode="min", factor=0.8, patience=10)
    keys = [(pk, kind, lk) for pk, o in model.skf_optimizers.items() for kind, pd in (("h", o.h_params),
                                                                                      ("s", o.s_params))
            for lk in pd]
    payload = {"tables_checksum": tables_checksum(tables), "table_seed": 4, "lr": TRAIN_LR,
               "struct_seed": struct_seed,
               "dos_target": np.stack([d.numpy() for d in dos_t]), "gap_target": np.array(gap_t),
               "param_keys": np.array(["|".join(k) for k in keys])}
    for i, st in enumerate(sts):
        for f in ("numbers", "positions", "cell", "kpoints"):
            payload[f"s{i}_{f}"] = np.asarray(st[f])
    orig = ref.utils._SymEigB.backward
    ref.utils._SymEigB.backward = staticmethod(_fixed_symeig_backward)
    try:
        for step in range(TRAIN_STEPS):
            opt.zero_grad()
            model.apply_constraints()
            losses, wsum = [], 0.0
            for st, d_t, g_t in zip(sts, dos_t, gap_t):
                dos, gap = _train_forward(model, st, sd)
                loss = torch.mean((dos - d_t) ** 2) + torch.abs(gap - g_t)
                w = float(len(st["numbers"]))
                losses.append(loss * w)
                wsum += w
            batch = sum(losses) / wsum
            reg = 1e-10 * sum(torch.sum(p ** 2) for p in model.parameters())
            total = batch + reg
            total.backward()
            torch.nn.utils.clip_grad_norm_(model.parameters(), max_norm=2.0)
            for (pk, kind, lk) in keys:             # the clipped gradient this step's AdamW update uses
                prm = getattr(model.skf_optimizers[pk], f"{kind}_params")[lk]
                payload[f"grad{step}|{pk}|{kind}|{lk}"] = prm.grad.detach().numpy().copy()
            opt.step()
            sched.step(total)
            payload[f"loss_{step}"] = float(total.detach())
            for (pk, kind, lk) in keys:
                prm = getattr(model.skf_optimizers[pk], f"{kind}_params")[lk]
                payload[f"step{step}|{pk}|{kind}|{lk}"] = prm.detach().numpy().copy()
            print(f"training step {step}: loss {float(total):.12e}")
    finally:
        ref.utils._SymEigB.backward = orig
    np.savez_compressed(os.path.join(HERE, "train_steps.npz"), **payload)


def fixture_energy_forces(name, st, shell_dict, table_seed, mesh):
    """get_energy / get_forces of compute_multi_element_properties (slakonet/optim.py:1066-1071):
    Fermi-smeared band energy (slakonet/main.py:1430-1448) and central-difference forces on the
    sum of eigenvalues at a 5x5x5 grid, delta = 0.01 Bohr (slakonet/main.py:198-281)."""
    zs = sorted({int(z) for z in st["numbers"]})
    full = syn.default_shell_dict()
    sd = {z: (shell_dict or full)[z] for z in zs}
    tables = syn.make_tables(zs, shell_dict or full, seed=table_seed)
    model = build_reference_model(ref, tables)
    geom = geometry(st)
    with torch.no_grad():
        props, ok = model.compute_multi_element_properties(geometry=geom, shell_dict=sd, kpoints=torch.tensor(mesh),
                                                           device="cpu", get_fermi=True, get_energy=True,
                                                           get_forces=True)
    payload = dict(numbers=st["numbers"], positions=st["positions"], cell=st["cell"], mesh=np.array(mesh),
                   table_seed=table_seed, tables_checksum=tables_checksum(tables), shell_z=np.array(zs),
                   shells=np.array([len(sd[z]) for z in zs]),
                   fermi_energy_Ha=float(props["fermi_energy_Ha"]),
                   eigenvalues=props["eigenvalues"][0].numpy(), k_weights=props["calc"].k_weights[0].numpy(),
                   total_energy=float(props["total_energy"]), forces=props["forces"][0].detach().numpy())
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **payload)
    print(name, "E", payload["total_energy"], "F", payload["forces"].round(6).tolist())


def fixtures_energy_forces():
    rng = np.random.default_rng(31)
    si = syn.diamond_si()
    si["positions"] = si["positions"] + rng.normal(0.0, 0.08, si["positions"].shape)
    fixture_energy_forces("ef_si", si, {14: [0, 1, 2]}, 0, (2, 2, 2))
    st = syn.random_structure(np.random.default_rng(32), 3, zmax=30)
    fixture_energy_forces("ef_rand", st, None, 4, (2, 2, 1))


def fixtures_pdos():
    si = syn.diamond_si()
    fixture_pdos("pdos_si", si, {14: [0, 1, 2]}, 0, (3, 3, 3))
    a = 5.65 * syn.ANGSTROM_TO_BOHR
    gaas = {"numbers": np.array([31, 33]), "positions": np.array([[0.0, 0.0, 0.0], [0.25 * a] * 3]),
            "cell": 0.5 * a * np.array([[0.0, 1.0, 1.0], [1.0, 0.0, 1.0], [1.0, 1.0, 0.0]])}
    fixture_pdos("pdos_gaas", gaas, None, 1, (3, 3, 3))
    # H (1 orbital) and Fe (9): 10 orbitals over 2 atoms; the reference splits them into equal blocks of 5
    hfe = {"numbers": np.array([1, 26]), "positions": np.array([[0.0, 0.0, 0.0], [1.6, 1.6, 1.6]]),
           "cell": np.eye(3) * 5.4}
    fixture_pdos("pdos_hfe", hfe, None, 2, (2, 2, 2))


if __name__ == "__main__":
    if "--gradients-only" in sys.argv:
        fixture_gradients()
        sys.exit(0)
    if "--pdos-only" in sys.argv:
        fixtures_pdos()
        sys.exit(0)
    if "--training-only" in sys.argv:
        fixture_training()
        sys.exit(0)
    if "--energy-forces-only" in sys.argv:
        fixtures_energy_forces()
        sys.exit(0)
    fixture_interp()
    fixture_blocks()
    fixture_fermi()
    fixture_si_cfg0()
    fixture_klines()
    fixture_random("rand_f4", 4, 5, 3, numbers=[1, 26, 60, 33], mesh=(2, 2, 3))
    fixture_random("rand_a", 6, 21, 21, zmax=30)
    fixture_random("rand_b", 9, 22, 22)
    fixture_random("rand_c", 3, 23, 23)
    fixture_gradients()
    fixtures_pdos()
    fixtures_energy_forces()
    fixture_training()
    print("golden fixtures written to", HERE)
