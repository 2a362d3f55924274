// Shared device helpers for the SlakoNet GB300 kernels.
//
// Complex numbers are double2 (x = real, y = imaginary).  On GB300 every
// FP64 instruction is expensive (about 1 TFLOP/s per GPU, and a warp FP64
// instruction costs the same with 1 or 32 active lanes), so helpers here keep
// FP64 work to fused multiply-adds and do sign flips and tests with integer
// operations on the bit patterns.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "../../include/slakonet_gb300.h"

#define SKN_DEVINL __device__ __forceinline__

SKN_DEVINL double flip_sign(double v) {
  return __longlong_as_double(__double_as_longlong(v) ^ (long long)0x8000000000000000ULL);
}
SKN_DEVINL double cond_flip(double v, bool flip) {
  return __longlong_as_double(__double_as_longlong(v) ^ (flip ? (long long)0x8000000000000000ULL : 0LL));
}
SKN_DEVINL bool is_zero_bits(double v) {
  return (__double_as_longlong(v) & 0x7fffffffffffffffLL) == 0;
}
SKN_DEVINL bool is_finite_bits(double v) {
  return ((__double_as_longlong(v) >> 52) & 0x7ff) != 0x7ff;
}

// c + a*b
SKN_DEVINL double2 cfma(double2 a, double2 b, double2 c) {
  c.x = fma(a.x, b.x, c.x);
  c.x = fma(-a.y, b.y, c.x);
  c.y = fma(a.x, b.y, c.y);
  c.y = fma(a.y, b.x, c.y);
  return c;
}
// c - a*conj(b)
SKN_DEVINL double2 cfms_conj(double2 a, double2 b, double2 c) {
  c.x = fma(-a.x, b.x, c.x);
  c.x = fma(-a.y, b.y, c.x);
  c.y = fma(-a.y, b.x, c.y);
  c.y = fma(a.x, b.y, c.y);
  return c;
}
// c + conj(a)*b
SKN_DEVINL double2 cfma_conj(double2 a, double2 b, double2 c) {
  c.x = fma(a.x, b.x, c.x);
  c.x = fma(a.y, b.y, c.x);
  c.y = fma(a.x, b.y, c.y);
  c.y = fma(-a.y, b.x, c.y);
  return c;
}
SKN_DEVINL double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
SKN_DEVINL double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }

// Block-wide sum of one double per thread; every thread gets the result.
// `red` needs blockDim.x/32 doubles; includes the barriers it needs.
SKN_DEVINL double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  for (int i = 0; i < nw; ++i) s += red[i];
  return s;
}

// Row/column of entry `e` in the packed column-major lower triangle
// (diagonal included) of an m x m matrix.  Column j starts at
// j*m - j*(j-1)/2.  FP32 estimate plus integer correction.
SKN_DEVINL void tri_index(int e, int m, int& i, int& j) {
  float b = 2.0f * (float)m + 1.0f;
  float disc = b * b - 8.0f * (float)e;
  int jj = (int)((b - sqrtf(fmaxf(disc, 0.0f))) * 0.5f);
  if (jj < 0) jj = 0;
  if (jj > m - 1) jj = m - 1;
  // offset(j) = j*m - j*(j-1)/2
  while (jj > 0 && (jj * m - (jj * (jj - 1)) / 2) > e) --jj;
  while (jj < m - 1 && ((jj + 1) * m - ((jj + 1) * jj) / 2) <= e) ++jj;
  j = jj;
  i = jj + (e - (jj * m - (jj * (jj - 1)) / 2));
}
