// Eigenvalues of a real symmetric tridiagonal matrix (diagonal d, squared
// off-diagonal e2, e2[i] coupling rows i and i+1), one eigenvalue per thread.
// Shared by the one-CTA and the cluster eigensolvers.
//
//  1. FP32 bisection on the rounded matrix brackets eigenvalue j to ~1e-6 of
//     the spectrum's scale (FP32 runs 64x faster than FP64 on GB300).
//  2. The bracket is widened by a margin covering the FP32 rounding and
//     checked with two FP64 Sturm counts (else the Gershgorin interval is used).
//  3. If it holds eigenvalue j alone, safeguarded Newton steps on the
//     characteristic polynomial p(x) = det(T - x I) finish it: p and p' come
//     from the three-term recurrence, each step also yields the Sturm count at
//     the new point, which keeps the bracket, and a step that leaves the bracket
//     is replaced by bisection.  Near a simple root Newton converges
//     quadratically, so 3-5 steps replace ~28 bisection steps.
//  4. Clustered or degenerate eigenvalues (the bracket holds several) are
//     bisected in FP64 to 1e-14 of the scale.
#pragma once
#include "skn_common.cuh"

namespace skn_sturm {
namespace {   // internal linkage: every including file gets its own copy

__device__ __forceinline__ int sign_bit(double v) { return (int)((unsigned long long)__double_as_longlong(v) >> 63); }

// Exponent field of |v| (biased), for power-of-two rescaling.
__device__ __forceinline__ int exp_field(double v) { return (int)((__double_as_longlong(v) >> 52) & 0x7ff); }

// Number of eigenvalues below x: sign changes of the determinant sequence
// p_i = (d_i - x) p_{i-1} - e2_{i-1} p_{i-2} (three FP64 operations per step, no
// division).  (p, p_prev) are rescaled by exact powers of two when p's exponent
// drifts, and an exact zero p_i takes the sign opposite to p_{i-1} (the tiny
// negative pivot LAPACK substitutes).
__device__ __forceinline__ int count64(const double* d, const double* e2, int n, double x) {
  double pm = 1.0, p = d[0] - x;
  if (is_zero_bits(p)) p = -0x1p-200;
  int c = sign_bit(p);
  int sp = c;
  for (int i = 1; i < n; ++i) {
    double pn = fma(-e2[i - 1], pm, (d[i] - x) * p);
    if (is_zero_bits(pn)) pn = flip_sign(p) * 0x1p-200;
    const int sn = sign_bit(pn);
    c += sn ^ sp;
    sp = sn;
    pm = p;
    p = pn;
    const int ex = exp_field(p);
    if (ex > 1023 + 480 || ex < 1023 - 480) {
      const double f = __longlong_as_double((long long)(2046 - ex) << 52);  // 2^(1023 - ex)
      p *= f;
      pm *= f;
    }
  }
  return c;
}

// The same count plus the Newton step p(x) / p'(x), from the recurrence and its
// derivative p'_i = (d_i - x) p'_{i-1} - p_{i-1} - e2_{i-1} p'_{i-2}; all four
// values share one power-of-two scale, so the ratio is unaffected.
__device__ __forceinline__ int count_newton64(const double* d, const double* e2, int n, double x, double& step) {
  double pm = 1.0, p = d[0] - x, dpm = 0.0, dp = -1.0;
  if (is_zero_bits(p)) p = -0x1p-200;
  int c = sign_bit(p);
  int sp = c;
  for (int i = 1; i < n; ++i) {
    const double t = d[i] - x;
    double pn = fma(-e2[i - 1], pm, t * p);
    const double dpn = fma(-e2[i - 1], dpm, fma(t, dp, -p));
    if (is_zero_bits(pn)) pn = flip_sign(p) * 0x1p-200;
    const int sn = sign_bit(pn);
    c += sn ^ sp;
    sp = sn;
    pm = p;
    p = pn;
    dpm = dp;
    dp = dpn;
    const int ex = max(exp_field(p), exp_field(dp));
    if (ex > 1023 + 480 || ex < 1023 - 480) {
      const double f = __longlong_as_double((long long)(2046 - ex) << 52);
      p *= f;
      pm *= f;
      dp *= f;
      dpm *= f;
    }
  }
  step = p / dp;
  return c;
}

// FP32 count on the rounded tridiagonal (LDL^T pivots; FP32 division is cheap).
__device__ __forceinline__ int count32(const float* d, const float* e2, int n, float x, float pivmin) {
  float q = d[0] - x;
  int c = q < 0.0f;
  for (int i = 1; i < n; ++i) {
    if (fabsf(q) < pivmin) q = -pivmin;
    q = (d[i] - x) - __fdiv_rn(e2[i - 1], q);
    c += q < 0.0f;
  }
  return c;
}

// Bounds shared by the threads of one matrix: Gershgorin interval [lo, hi]
// (already widened), FP64 target width atol, FP32 pivot floor, FP32 margin.
struct Bounds {
  double lo, hi, atol, margin;
  float pivmin32;
};

__device__ __forceinline__ Bounds make_bounds(double lo, double hi, double emax, int n) {
  Bounds B;
  const double bnorm = fmax(fmax(fabs(lo), fabs(hi)), 1e-300);
  B.lo = lo - (2.2e-16 * bnorm * 4.0 * n + 1e-300);
  B.hi = hi + (2.2e-16 * bnorm * 4.0 * n + 1e-300);
  B.atol = 1e-14 * bnorm;
  B.pivmin32 = 1.1754944e-38f * fmaxf(1.0f, (float)emax);
  B.margin = 32.0 * 5.9604645e-8 * bnorm;   // covers FP32 rounding of T and of the count
  return B;
}

// Eigenvalue j (0-based, ascending) of the tridiagonal.
__device__ double eigenvalue(const double* d, const double* e2, const float* d32, const float* e232, int n, int j,
                             const Bounds& B) {
  float a32 = (float)B.lo, b32 = (float)B.hi;
  for (int it = 0; it < 40; ++it) {
    const float mid = 0.5f * (a32 + b32);
    if (!(mid > a32 && mid < b32)) break;
    if (count32(d32, e232, n, mid, B.pivmin32) > j) b32 = mid; else a32 = mid;
  }
  double a = (double)a32 - B.margin, b = (double)b32 + B.margin;
  if (a < B.lo) a = B.lo;
  if (b > B.hi) b = B.hi;
  const int ca = count64(d, e2, n, a);
  const int cb = count64(d, e2, n, b);
  if (!(ca <= j && cb > j)) {
    a = B.lo;
    b = B.hi;
  } else if (ca == j && cb == j + 1) {
    // eigenvalue j alone in (a, b]: safeguarded Newton from the FP32 estimate.  A step
    // that leaves the bracket, or is not at least halving the previous step, is
    // replaced by bisection, so the bracket keeps shrinking.
    double x = 0.5 * ((double)a32 + (double)b32);
    if (!(x > a && x < b)) x = 0.5 * (a + b);
    double dx_old = b - a;
    for (int it = 0; it < 16; ++it) {
      double step;
      const int c = count_newton64(d, e2, n, x, step);
      if (c > j) b = x; else a = x;
      if (b - a <= B.atol) break;
      const double xn = x - step;
      // converged: the last step may land on the bracket's edge (the root lies within rounding of
      // the point just counted), so it is tested before the bracket, not after
      if (fabs(step) <= B.atol && xn >= a && xn <= b) return xn;
      if (xn > a && xn < b && fabs(step) <= 0.5 * dx_old) {
        dx_old = fabs(step);
        x = xn;
      } else {
        dx_old = 0.5 * (b - a);
        x = 0.5 * (a + b);
      }
    }
  }
  for (int it = 0; it < 200 && (b - a) > B.atol; ++it) {
    const double mid = 0.5 * (a + b);
    if (mid <= a || mid >= b) break;
    if (count64(d, e2, n, mid) > j) b = mid; else a = mid;
  }
  return 0.5 * (a + b);
}

}  // namespace
}  // namespace skn_sturm
