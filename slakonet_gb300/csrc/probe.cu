// FP64 throughput probes: the roofline denominator for the FP64-bound kernels.
//
// k_fp64_fma: every thread runs 8 independent fused multiply-add chains, so
// the FP64 pipe (not latency) bounds the kernel; flops = 2 * 8 * iters * threads.
// k_fp64_dmma: every warp runs 8 independent chains of the FP64 tensor
// instruction mma.sync.m8n8k4.f64 (D = A B + C, 8x8x4); flops = 2*8*8*4 per
// instruction = 512 * 8 * iters * warps.  Comparing the two rates shows whether
// the FP64 tensor path is faster than plain FMAs on this GPU.
#include "skn_common.cuh"

namespace {
__global__ void k_fp64_fma(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * (int64_t)blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void k_fp64_dmma(double* out, int iters, double a, double b) {
  double c0[8], c1[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    c0[q] = 1e-3 * (threadIdx.x + q);
    c1[q] = 2e-3 * (threadIdx.x + q);
  }
  const double av = a * (1.0 + 1e-3 * (threadIdx.x & 31)), bv = b;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int q = 0; q < 8; ++q)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                   : "+d"(c0[q]), "+d"(c1[q])
                   : "d"(av), "d"(bv));
  }
  double t = 0.0;
#pragma unroll
  for (int q = 0; q < 8; ++q) t += c0[q] + c1[q];
  out[blockIdx.x * (int64_t)blockDim.x + threadIdx.x] = t;
}
}  // namespace

extern "C" int skn_fp64_probe_dmma(double* out, int blocks, int iters, cudaStream_t stream) {
  if (!out || blocks <= 0 || iters <= 0) return SKN_ERR_ARG;
  k_fp64_dmma<<<blocks, 256, 0, stream>>>(out, iters, 1e-4, 1e-4);
  return cudaPeekAtLastError() == cudaSuccess ? SKN_OK : SKN_ERR_CUDA;
}

extern "C" int skn_fp64_probe(double* out, int blocks, int iters, cudaStream_t stream) {
  if (!out || blocks <= 0 || iters <= 0) return SKN_ERR_ARG;
  k_fp64_fma<<<blocks, 256, 0, stream>>>(out, iters, 0.999999, 1e-7);
  return cudaPeekAtLastError() == cudaSuccess ? SKN_OK : SKN_ERR_CUDA;
}
