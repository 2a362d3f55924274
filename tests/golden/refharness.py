"""Import harness for the reference SlakoNet package (fixture generation only).

This module is used by ``make_golden.py`` in a container that holds a
checkout of the reference; ``SLAKONET_REF`` names its directory (the one that
contains the ``slakonet`` package).  The library and the
GPU tests never import it: the reference source tree does not exist on the
GPU hosts, and the committed golden fixtures are what travels.  The one other
user is ``bench.py --reference-gpu``, which points ``REF_ROOT`` at a pip
installation of the reference in ``baseline/_ref`` (when present) to time the
reference's own per-structure GPU path.

The reference imports ``ase``, ``jarvis`` and ``matplotlib`` at module level
(slakonet/main.py:4-20, slakonet/optim.py:19-36).  None of them is on the
compute path this project replaces, so lightweight stand-ins are placed in
``sys.modules`` before the reference is imported.  The only function the path
needs from them is ``jarvis.core.specie.atomic_numbers_to_symbols``, used by
the model's atomic-number -> symbol map (slakonet/optim.py:162-164); the
stand-in maps through the reference's own ``slakonet.elements`` table.
"""
import os
import sys
import types

# Directory holding the reference's ``slakonet`` package: $SLAKONET_REF, else the pip installation
# of the reference in baseline/_ref beside this repository's root.
REF_ROOT = os.environ.get("SLAKONET_REF") or os.path.join(
    os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))), "baseline", "_ref")


def _install_stubs():
    if "jarvis" in sys.modules and getattr(sys.modules["jarvis"], "_skn_stub", False):
        return

    def mod(name):
        m = types.ModuleType(name)
        m._skn_stub = True
        sys.modules[name] = m
        return m

    class _Anything:
        def __init__(self, *a, **k):
            pass

        def __getattr__(self, item):
            return _Anything()

        def __call__(self, *a, **k):
            return _Anything()

    ase = mod("ase")
    ase.Atoms = _Anything
    ase_io = mod("ase.io")
    ase.io = ase_io
    mpl = mod("matplotlib")
    mpl.rcParams = {}
    mpl.use = lambda *a, **k: None
    plt = mod("matplotlib.pyplot")
    mpl.pyplot = plt
    plt.rcParams = {}
    gs = mod("matplotlib.gridspec")
    gs.GridSpec = _Anything
    mpl.gridspec = gs
    for nm in ("figure", "plot", "savefig", "close", "subplots", "xlabel", "ylabel",
               "legend", "tight_layout", "title", "xlim", "ylim", "axhline", "axvline"):
        setattr(plt, nm, lambda *a, **k: _Anything())
    jarvis = mod("jarvis")
    core = mod("jarvis.core")
    jarvis.core = core
    atoms = mod("jarvis.core.atoms")
    atoms.Atoms = _Anything
    kp = mod("jarvis.core.kpoints")
    kp.Kpoints3D = _Anything
    specie = mod("jarvis.core.specie")
    db = mod("jarvis.db")
    fig = mod("jarvis.db.figshare")
    fig.data = lambda *a, **k: []
    io_ = mod("jarvis.io")
    vasp = mod("jarvis.io.vasp")
    outs = mod("jarvis.io.vasp.outputs")
    outs.Vasprun = _Anything
    inputs = mod("jarvis.io.vasp.inputs")
    inputs.Poscar = _Anything

    def atomic_numbers_to_symbols(zz):
        from slakonet.elements import chemical_symbols
        return [chemical_symbols[int(z)] for z in zz]

    specie.atomic_numbers_to_symbols = atomic_numbers_to_symbols


def import_reference():
    """Return the reference modules (optim, main, skf, atoms, slaterkoster, ...)."""
    _install_stubs()
    if REF_ROOT not in sys.path:
        sys.path.insert(0, REF_ROOT)
    import slakonet.optim as optim
    import slakonet.main as main
    import slakonet.skf as skf
    import slakonet.atoms as atoms
    import slakonet.slaterkoster as sk
    import slakonet.interpolation as interp
    import slakonet.fermi as fermi
    import slakonet.utils as utils
    import slakonet.predict_slakonet as predict
    return types.SimpleNamespace(optim=optim, main=main, skf=skf, atoms=atoms,
                                 sk=sk, interp=interp, fermi=fermi, utils=utils, predict=predict)


def build_reference_model(ref, tables):
    """Build a ``MultiElementSkfParameterOptimizer`` from synthetic tables.

    Follows the construction in ``load_ultra_compact`` (slakonet/optim.py:552-620):
    an instance made with ``__new__``, one ``SkfParameterOptimizer`` per
    element pair holding ``h_params`` / ``s_params`` ParameterDicts.
    ``tables`` is the dict produced by ``slakonet_gb300.synthetic``.
    """
    import torch
    import torch.nn as nn
    from slakonet.elements import chemical_symbols

    M = ref.optim.MultiElementSkfParameterOptimizer
    P = ref.optim.SkfParameterOptimizer
    inst = M.__new__(M)
    nn.Module.__init__(inst)
    zz = list(range(1, 100))
    inst.atomic_num_to_symbol = {z: chemical_symbols[z] for z in zz}
    inst.skf_optimizers = nn.ModuleDict()
    grid = tables["grid"]
    for (za, zb), pair in tables["pairs"].items():
        key = f"{chemical_symbols[za]}-{chemical_symbols[zb]}"
        opt = P.__new__(P)
        nn.Module.__init__(opt)
        h = {f"{l1}-{l2}": torch.tensor(v, dtype=torch.float64) for (l1, l2), v in pair["H"].items()}
        s = {f"{l1}-{l2}": torch.tensor(v, dtype=torch.float64) for (l1, l2), v in pair["S"].items()}
        skf_dict = {
            "atom_pair": [za, zb],
            "hamiltonian": h,
            "overlap": s,
            "grid": [float(g) for g in grid],
            "hs_cutoff": float(grid[-1]),
            "atomic": za == zb,
        }
        if za == zb:
            el = tables["elements"][za]
            skf_dict["atomic_data"] = {
                "on_sites": [float(x) for x in el["on_sites"]],
                "hubbard_us": [0.0] * len(el["on_sites"]),
                "mass": 1.0,
                "occupations": [float(x) for x in el["occupations"]],
            }
        opt.skf_dict = skf_dict
        opt.h_params = nn.ParameterDict({k: nn.Parameter(v.clone()) for k, v in h.items()})
        opt.s_params = nn.ParameterDict({k: nn.Parameter(v.clone()) for k, v in s.items()})
        opt.grid = skf_dict["grid"]
        opt.atomic_data = skf_dict.get("atomic_data")
        opt.atom_pair = skf_dict["atom_pair"]
        opt.hs_cutoff = skf_dict["hs_cutoff"]
        inst.skf_optimizers[key] = opt
    return inst
