"""The device-wide eigensolver with its rank-2k updates on the tensor cores (skn_eigh_gen_wide_tc).

The emulated FP64 updates (7 integer bf16 slices of 7 bits per operand row, exact FP32 accumulation per
slice level in TMEM) must give eigenvalues within 1e-8 eV of LAPACK and of the FP64 path, on complex and
real problems, at sizes where the trailing matrices cross the 512-row threshold and leave partial tiles,
and a problem's results must not depend on its group.
"""
import numpy as np
import pytest
import scipy.linalg as sla
import torch

from test_gpu_wide import _pairs, _wide
from slakonet_gb300._lib import call, ptr

pytestmark = pytest.mark.gpu
H2E = 27.211


def _wide_tc(Hs, Ss, real=False, slots=None):
    import ctypes
    from test_gpu_wide import DEV, _pack
    n = Hs[0].shape[0]
    count = len(Hs)
    nv = torch.full((count,), n, dtype=torch.int32, device=DEV)
    off = torch.arange(count, dtype=torch.int64, device=DEV) * n * n
    eo = torch.arange(count, dtype=torch.int64, device=DEV) * n
    prob = torch.as_tensor(np.arange(count) if slots is None else np.asarray(slots), dtype=torch.int32, device=DEV)
    H, S = _pack(Hs), _pack(Ss)
    eig = torch.full((count * n,), -7.0, dtype=torch.float64, device=DEV)
    st = torch.full((count,), -1, dtype=torch.int32, device=DEV)
    need = ctypes.c_int64(0)
    call("skn_eigh_wide_scratch_bytes", len(prob), n, ctypes.addressof(need))
    scratch = torch.empty(need.value // 8, dtype=torch.float64, device=DEV)
    call("skn_eigh_gen_wide_tc", len(prob), n, ptr(prob), ptr(nv), ptr(off), ptr(eo), ptr(H), ptr(S), ptr(eig),
         ptr(st), ptr(scratch), need.value, int(real), torch.cuda.current_stream(DEV).cuda_stream)
    torch.cuda.synchronize(DEV)
    return eig.cpu().numpy().reshape(count, n), st.cpu().numpy()


@pytest.mark.parametrize("n,real", [(545, False), (700, False), (1100, False), (600, True), (1030, True)])
def test_tensor_core_updates_agree_with_lapack_and_fp64_path(n, real):
    Hs, Ss = _pairs(n, 2, seed=500 + n, real=real)
    got, st = _wide_tc(Hs, Ss, real=real)
    ref, st_ref = _wide(Hs, Ss, real=real)
    assert (st == 0).all() and (st_ref == 0).all()
    lap = [sla.eigh(Hs[i].real if real else Hs[i], Ss[i].real if real else Ss[i], eigvals_only=True) for i in range(2)]
    d_lapack = max(np.abs(got[i] - lap[i]).max() for i in range(2)) * H2E
    d_fp64 = np.abs(got - ref).max() * H2E
    print(f"n = {n} {'real' if real else 'complex'}: tensor-core path vs LAPACK {d_lapack:.1e} eV, "
          f"vs FP64 path {d_fp64:.1e} eV")
    assert d_lapack <= 1e-8 and d_fp64 <= 1e-8


def test_tensor_core_results_do_not_depend_on_the_group():
    Hs, Ss = _pairs(600, 3, seed=77)
    together, _ = _wide_tc(Hs, Ss, slots=[2, 0, 1])
    for i in range(3):
        alone, st = _wide_tc([Hs[i]], [Ss[i]])
        assert st[0] == 0
        assert np.array_equal(alone[0], together[i]), i
