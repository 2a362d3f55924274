"""ctypes binding of the C ABI in ``include/slakonet_gb300.h``.

The library is loaded from the package directory (built in-tree by
``slakonet_gb300.build``).  There is no fallback: every compute call goes to
the CUDA library, and a missing library or a non-zero status raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

_LIB = None
_LOAD_LOCK = threading.Lock()   # server workers can make their first call at the same time

SKN_OK = 0
SKN_ERR_ARG = 1
SKN_ERR_NOT_SPD = 2
SKN_ERR_NAN = 3
SKN_ERR_NO_CONVERGE = 4
SKN_ERR_CAPACITY = 5
SKN_ERR_CUDA = 6
SKN_NSTAT = 24

_ERRS = {1: "invalid argument", 2: "not positive definite", 3: "NaN", 4: "no convergence",
         5: "capacity exceeded", 6: "CUDA launch/runtime failure"}

P = C.c_void_p
I32 = C.c_int32
I64 = C.c_int64
F64 = C.c_double

# name -> argtypes (every function returns int)
SIGNATURES = {
    "skn_abi_version": [],
    "skn_bond_counts": [I32, I64, P, P, P, P, F64, P, P, P],
    "skn_bond_fill": [I32, I64, P, P, P, P, F64, P, P, P, P, P, P, P, P, P, P, P],
    "skn_image_phases": [I32, P, P, P, P, P, P],
    "skn_sk_blocks": [I64, P, P, P, P, P, P, I32, P, P, P, P, P, P, P, P, P, P, P, P, P],
    "skn_bloch": [I32, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, I32, P, P, P],
    "skn_bloch_pairs": [I32, I64, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, I32, P, P, P],
    "skn_eigh_gen_batched": [I32, P, P, P, P, P, P, P, P, P, I32, P],
    "skn_eigh_gen_batched_real": [I32, P, P, P, P, P, P, P, P, P, I32, P],
    "skn_fermi_gap": [I32, P, P, P, P, P, P, P, F64, F64, I32, P, P, P, P],
    "skn_dos": [I32, P, P, P, P, P, P, P, F64, F64, I32, F64, F64, P, P, P, P],
    "skn_fp64_probe": [P, I32, I32, P],
    "skn_fp64_probe_dmma": [P, I32, I32, P],
    "skn_tc_gemm_bf16": [P, P, P, I32, I32, I32, P, P],
    "skn_gemm_f64_emulated": [P, P, P, I32, I32, I32, I32, P, I64, P, P],
    "skn_gemm_f64_emulated_scratch_bytes": [I32, I32, I32, I32, P],
    "skn_eigh_gen_vectors": [I32, P, P, P, P, P, P, P, P, P, P, P, I64, P, I32, P],
    "skn_eigh_vectors_scratch_bytes": [I32, I32, P],
    "skn_eigh_gen_vectors_noalloc": [I32, P, P, P, P, P, P, P, P, P, I64, I32, P],
    "skn_eigh_gen_large": [I32, P, P, P, P, P, P, P, P, P, P, I64, I32, I32, P],
    "skn_eigh_large_scratch_bytes": [I32, I32, I32, P],
    "skn_eigh_gen_wide": [I32, I32, P, P, P, P, P, P, P, P, P, I64, I32, P],
    "skn_eigh_wide_scratch_bytes": [I32, I32, P],
    "skn_eigh_gen_wide_tc": [I32, I32, P, P, P, P, P, P, P, P, P, I64, I32, P],
    "skn_adj_projectors": [I32, P, P, P, P, P, P, P, P, P, P],
    "skn_adj_bloch": [I64] + [P] * 18 + [P],
    "skn_adj_tables": [I64, P, P, P, P, P, P, I32, P, P, P, P, P, P, P, P, P, P, P, P],
    "skn_dos_backward": [I32, P, P, P, P, P, P, P, F64, F64, I32, F64, F64, P, P, I32, P],
    "skn_atom_pdos": [I32, I32, I32, P, P, P, I32, F64, F64, F64, I32, F64, F64, P, P, P, P],
}
for _sfx in ("_t32", "_t64", "_t256", "_blk"):
    SIGNATURES["skn_eigh_gen_batched" + _sfx] = SIGNATURES["skn_eigh_gen_batched"]
    SIGNATURES["skn_eigh_gen_batched_real" + _sfx] = SIGNATURES["skn_eigh_gen_batched"]
    SIGNATURES["skn_eigh_gen_vectors" + _sfx] = SIGNATURES["skn_eigh_gen_vectors"]
    SIGNATURES["skn_eigh_vectors_scratch_bytes" + _sfx] = SIGNATURES["skn_eigh_vectors_scratch_bytes"]


class SknError(RuntimeError):
    pass


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building first if needed) and return the ctypes library."""
    global _LIB
    if _LIB is not None:
        return _LIB
    with _LOAD_LOCK:
        if _LIB is not None:
            return _LIB
        path = lib_path()
        if not os.path.exists(path) or _build._stale():
            if not build_if_missing:
                raise SknError(f"CUDA library not built: {path}")
            _build.build()
        lib = C.CDLL(path)
        for name, argt in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = argt
            fn.restype = C.c_int
        _LIB = lib
        return lib


def call(name: str, *args):
    rc = getattr(load(), name)(*args)
    if rc != SKN_OK:
        raise SknError(f"{name} returned {rc} ({_ERRS.get(rc, 'unknown')})")
    return rc


def ptr(t) -> int:
    """Device (or host) address of a torch tensor, 0 for None."""
    return 0 if t is None else int(t.data_ptr())
