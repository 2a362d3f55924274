"""bf16 tensor-core GEMM (tcgen05) and the FP64 GEMM emulated on it (needs a GB300).

1. Exactness of the FP32 accumulator: integer operands of at most 8 significant
   bits (|a|, |b| <= 256, held exactly in bf16) with K <= 256 keep every
   product and partial sum an integer below 2^24.  The tensor-core result must
   equal the exact integer product bit for bit, for random operands and for
   sums that cancel from large partial values.
2. The FP64 emulation (7 integer slices per operand row, slice products summed
   in FP64) must agree with an FP64 GEMM to FP64 rounding: every entry within
   2^-50 of sum_k |A_ik| |B_jk|.
"""
import ctypes

import numpy as np
import pytest
import torch

from slakonet_gb300 import _lib
from slakonet_gb300._lib import call, ptr

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _bf16_bits(x: np.ndarray) -> torch.Tensor:
    t = torch.tensor(x, dtype=torch.float32).to(torch.bfloat16)
    assert torch.equal(t.float(), torch.tensor(x, dtype=torch.float32)), "operand not exact in bf16"
    return t.view(torch.int16).to(DEV).contiguous()


def _tc(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    M, K = a.shape
    N = b.shape[0]
    A, B = _bf16_bits(a), _bf16_bits(b)
    D = torch.full((M, N), np.nan, dtype=torch.float32, device=DEV)
    err = torch.zeros(1, dtype=torch.int32, device=DEV)
    call("skn_tc_gemm_bf16", ptr(A), ptr(B), ptr(D), M, N, K, ptr(err), torch.cuda.current_stream(DEV).cuda_stream)
    torch.cuda.synchronize(DEV)
    assert int(err.item()) == 0
    return D.cpu().numpy()


@pytest.mark.parametrize("K", [64, 256])
def test_integer_slices_accumulate_exactly(K):
    rng = np.random.default_rng(K)
    a = rng.integers(-256, 257, size=(256, K)).astype(np.int64)
    b = rng.integers(-256, 257, size=(128, K)).astype(np.int64)
    exact = a @ b.T
    assert np.abs(exact).max() < 2 ** 24 and np.abs(np.cumsum(a[:, None, :] * b[None, :, :], -1)).max() < 2 ** 24
    d = _tc(a.astype(np.float64), b.astype(np.float64))
    bad = int((d.astype(np.int64) != exact).sum()) + int((d != np.round(d)).sum())
    print(f"K={K}: {exact.size} dot products of random integer slices, {bad} inexact")
    assert bad == 0


def test_cancelling_large_partial_sums_stay_exact():
    """Rows whose products alternate +-2^16 with odd small terms between: partial sums reach 2^23 while the
    result is small, and mixed magnitudes meet inside every 16-wide MMA step."""
    K = 256
    rng = np.random.default_rng(7)
    a = np.zeros((128, K))
    b = np.zeros((128, K))
    for i in range(128):
        big = rng.permutation(K)[: K // 2]
        a[i] = rng.integers(-3, 4, size=K)
        a[i, big] = 256 * rng.choice([-1, 1], size=len(big))
    for j in range(128):
        b[j] = rng.integers(-255, 256, size=K)
        b[j, :: 2] = 256
    exact = a.astype(np.int64) @ b.astype(np.int64).T
    partial = np.abs(np.cumsum(a[:, None, :].astype(np.int64) * b[None, :, :].astype(np.int64), -1)).max()
    assert partial < 2 ** 24
    d = _tc(a, b)
    bad = int((d.astype(np.int64) != exact).sum())
    print(f"cancelling sums: partial sums up to {partial:.3e}, {bad} of {exact.size} inexact")
    assert bad == 0


def _emulated(A: torch.Tensor, B: torch.Tensor, slices=7):
    M, K = A.shape
    N = B.shape[0]
    need = ctypes.c_int64(0)
    call("skn_gemm_f64_emulated_scratch_bytes", M, N, K, slices, ctypes.addressof(need))
    scratch = torch.empty(need.value, dtype=torch.uint8, device=DEV)
    C = torch.empty(M, N, dtype=torch.float64, device=DEV)
    err = torch.zeros(1, dtype=torch.int32, device=DEV)
    call("skn_gemm_f64_emulated", ptr(A), ptr(B), ptr(C), M, N, K, slices, ptr(scratch), need.value, ptr(err),
         torch.cuda.current_stream(DEV).cuda_stream)
    torch.cuda.synchronize(DEV)
    assert int(err.item()) == 0
    return C


def test_emulated_fp64_gemm_matches_fp64():
    rng = np.random.default_rng(3)
    M, N, K = 256, 384, 512
    a = rng.standard_normal((M, K)) * 10.0 ** rng.uniform(-3, 3, size=(M, 1))
    b = rng.standard_normal((N, K)) * 10.0 ** rng.uniform(-3, 3, size=(N, 1))
    a[:, ::5] *= 1e-6                                  # spread of magnitudes inside each row
    A = torch.tensor(a, device=DEV)
    B = torch.tensor(b, device=DEV)
    C = _emulated(A, B).cpu().numpy()
    ref = a @ b.T
    bound = np.abs(a) @ np.abs(b).T
    rel = float((np.abs(C - ref) / bound).max())
    print(f"emulated FP64 GEMM {M}x{N}x{K}, 7 slices: max |C - C_fp64| / (|A||B|^T) = {rel:.2e} (2^-52 = 2.2e-16)")
    assert rel <= 2.0 ** -50


def test_emulated_fp64_gemm_rate():
    """Rate of the emulation at M = N = 2048, K = 1024 (FP64-equivalent TFLOP/s), beside torch's FP64 GEMM."""
    M = N = 2048
    K = 1024
    g = torch.Generator(device=DEV).manual_seed(0)
    A = torch.randn(M, K, dtype=torch.float64, device=DEV, generator=g)
    B = torch.randn(N, K, dtype=torch.float64, device=DEV, generator=g)
    _emulated(A, B)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    ev[0].record()
    C = _emulated(A, B)
    ev[1].record()
    ev[2].record()
    ref = A @ B.T
    ev[3].record()
    torch.cuda.synchronize(DEV)
    t_em = ev[0].elapsed_time(ev[1]) * 1e-3
    t_64 = ev[2].elapsed_time(ev[3]) * 1e-3
    fl = 2.0 * M * N * K
    rel = float(((C - ref).abs() / (A.abs() @ B.abs().T)).max())
    print(f"emulated FP64 GEMM {M}x{N}x{K}: {fl / t_em / 1e12:.2f} TFLOP/s (28 slice products); torch FP64 GEMM "
          f"{fl / t_64 / 1e12:.2f} TFLOP/s; max rel {rel:.1e}")
    assert rel <= 2.0 ** -50
