"""Atom-type projected DOS on the GPU.

``compute_atom_projected_dos`` keeps the signature, inputs and return value of
the reference's function (slakonet/predict_slakonet.py:119-210): it takes the
properties dict of ``compute_multi_element_properties(..., with_eigenvectors=True,
get_fermi=True)`` and the geometry, and returns the energy grid (eV relative to
E_F), a dict of per-atom-type PDOS arrays and the atom types in first-seen
order.  As in the reference, the orbitals are split into equal contiguous
blocks, one per atom, and an atom type's weight for a band is the sum of
|c_i|^2 over its blocks; the sum over (k, band) runs in the CUDA kernel
``skn_atom_pdos`` instead of a Python double loop.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from ._lib import call, ptr
from .elements import SYMBOLS

H2E = 27.211


def _atom_types(geometry):
    syms = getattr(geometry, "chemical_symbols", None)
    if syms is not None:
        return list(syms[0])
    z = torch.as_tensor(geometry.atomic_numbers).reshape(-1).tolist()
    return [SYMBOLS[int(a)] for a in z]


def compute_atom_projected_dos(properties, geometry, sigma=0.1, energy_range=(-8, 6), filename="slakonet_bands.png",
                               n_points: int = 1000):
    fermi_ev = float(properties["fermi_energy_eV"])
    calc = properties["calc"]
    ev = calc.eigenvectors                       # [1, n_orb, nb, nk]
    eig = torch.as_tensor(calc.eigenvalue)       # [1, nk, nb], Hartree
    dev = ev.device if ev.is_cuda else torch.device("cuda")
    atom_types = _atom_types(geometry)
    unique = list(dict.fromkeys(atom_types))
    n_orb = int(ev.shape[1])
    n_atoms = len(atom_types)
    if n_orb % n_atoms != 0:
        raise ValueError(f"n_orbitals ({n_orb}) not divisible by n_atoms ({n_atoms}).")
    per = n_orb // n_atoms
    group = np.repeat(np.array([unique.index(a) for a in atom_types], dtype=np.int32), per)
    nk, nb = int(eig.shape[1]), int(eig.shape[2])
    if eig.dim() != 3 or tuple(ev.shape) != (1, n_orb, nb, nk):
        # the kernel indexes the eigenvectors with the eigenvalue array's sizes
        raise ValueError(f"eigenvectors {tuple(ev.shape)} do not match eigenvalues {tuple(eig.shape)}: "
                         f"expected [1, n_orbitals, n_bands, n_kpoints] = [1, {n_orb}, {nb}, {nk}]")
    _lib.load()
    with torch.cuda.device(dev):
        vec = ev[0].permute(2, 0, 1).to(device=dev, dtype=torch.complex128).contiguous()   # [nk, n_orb, nb]
        e = eig[0].to(device=dev, dtype=torch.float64).contiguous()
        grp = torch.as_tensor(group, device=dev)
        weights = torch.empty(max(nk * nb * len(unique), 1), dtype=torch.float64, device=dev)
        grid = torch.empty(n_points, dtype=torch.float64, device=dev)
        pdos = torch.empty(len(unique) * n_points, dtype=torch.float64, device=dev)
        stream = torch.cuda.current_stream(dev).cuda_stream
        call("skn_atom_pdos", nk, nb, n_orb, ptr(e), ptr(torch.view_as_real(vec)), ptr(grp), len(unique), fermi_ev,
             float(energy_range[0]), float(energy_range[1]), int(n_points), float(sigma), H2E, ptr(weights),
             ptr(grid), ptr(pdos), stream)
        grid_h = grid.cpu().numpy()
        pdos_h = pdos.view(len(unique), n_points).cpu().numpy()
    return grid_h, {a: pdos_h[i] for i, a in enumerate(unique)}, unique
