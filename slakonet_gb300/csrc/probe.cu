// FP64 throughput probe: the roofline denominator for the FP64-bound kernels.
//
// Every thread runs 8 independent fused multiply-add chains, so the FP64
// pipe (not latency) bounds the kernel; flops = 2 * 8 * iters * threads.
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
}  // namespace

extern "C" int skn_fp64_probe(double* out, int blocks, int iters, cudaStream_t stream) {
  if (!out || blocks <= 0 || iters <= 0) return SKN_ERR_ARG;
  k_fp64_fma<<<blocks, 256, 0, stream>>>(out, iters, 0.999999, 1e-7);
  return cudaPeekAtLastError() == cudaSuccess ? SKN_OK : SKN_ERR_CUDA;
}
