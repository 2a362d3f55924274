// Device helpers shared by the forward Slater-Koster block kernel and its
// adjoint: real-harmonic rotation matrices of a bond direction and the
// reference's 8-point spline window (Lagrange weights, exact tail).
#pragma once
#include "skn_common.cuh"
#include "rot_coeffs.cuh"

namespace {

constexpr int WARP_SMEM = 152;  // doubles per warp: D0[1] D1[9] D2[25] D3[49] VH[32] VS[32] + pad

__device__ __forceinline__ double rot_get(const double* D, int l, int row, int col) {
  // row, col in -l..l
  return D[(row + l) * (2 * l + 1) + (col + l)];
}

// P(i, l, a, b) of the recursion: one D^1 entry times one D^(l-1) entry (two where |b| == l).
__device__ __forceinline__ double rot_P(const double* R1, const double* Rl1, int l, int i, int a, int b) {
  const int lm = l - 1;
  a = a < -lm ? -lm : (a > lm ? lm : a);  // rows outside D^(l-1) only occur with zero weight
  if (b == l)
    return fma(rot_get(R1, 1, i, 1), rot_get(Rl1, lm, a, lm), -rot_get(R1, 1, i, -1) * rot_get(Rl1, lm, a, -lm));
  if (b == -l)
    return fma(rot_get(R1, 1, i, 1), rot_get(Rl1, lm, a, -lm), rot_get(R1, 1, i, -1) * rot_get(Rl1, lm, a, lm));
  return rot_get(R1, 1, i, 0) * rot_get(Rl1, lm, a, b);
}

__device__ __forceinline__ double rot_entry(int l, int e, const double* R1, const double* Rl1) {
  const int w = 2 * l + 1;
  const int m = e / w - l, n = e % w - l;
  const double* c = SKN_ROT_W + 5 * (SKN_ROT_OFF[l] + e);
  double pu = rot_P(R1, Rl1, l, 0, m, n);
  double pv1, pv2, pw1, pw2;
  if (m == 0) {
    pv1 = rot_P(R1, Rl1, l, 1, 1, n);
    pv2 = rot_P(R1, Rl1, l, -1, -1, n);
    pw1 = 0.0;
    pw2 = 0.0;
  } else if (m > 0) {
    pv1 = rot_P(R1, Rl1, l, 1, m - 1, n);
    pv2 = rot_P(R1, Rl1, l, -1, -m + 1, n);
    pw1 = rot_P(R1, Rl1, l, 1, m + 1, n);
    pw2 = rot_P(R1, Rl1, l, -1, -m - 1, n);
  } else {
    pv1 = rot_P(R1, Rl1, l, 1, m + 1, n);
    pv2 = rot_P(R1, Rl1, l, -1, -m - 1, n);
    pw1 = rot_P(R1, Rl1, l, 1, m - 1, n);
    pw2 = rot_P(R1, Rl1, l, -1, -m + 1, n);
  }
  double v = c[0] * pu;
  v = fma(c[1], pv1, v);
  v = fma(c[2], pv2, v);
  v = fma(c[3], pw1, v);
  v = fma(c[4], pw2, v);
  return v;
}

// Reference Neville recursion (first-point start, always adding c[0]) with
// uncontracted IEEE operations, for the tail's finite differences.
__device__ double neville8_exact(const double* xa, const double* ya, double r) {
  double c[8], d[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) { c[k] = ya[k]; d[k] = ya[k]; }
  double y = ya[0];
  for (int mm = 0; mm < 7; ++mm) {
    for (int ii = 0; ii < 7 - mm; ++ii) {
      double r0 = __dsub_rn(xa[ii], xa[ii + mm + 1]);
      double r1 = __ddiv_rn(__dsub_rn(c[ii + 1], d[ii]), r0);
      c[ii] = __dmul_rn(__dsub_rn(xa[ii], r), r1);
      d[ii] = __dmul_rn(__dsub_rn(xa[ii + mm + 1], r), r1);
    }
    y = __dadd_rn(y, c[0]);
  }
  return y;
}

// Tail value from the last eight table values yb = row[ng-9 .. ng-2]
// (slakonet/interpolation.py:173-236, 241-252).  Linear in yb.
__device__ double tail_value8(const double* yb, int ng, double h, double r) {
  const double tail = 1.0, delta = 1e-5;
  double xa[8], ya[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    xa[k] = __dmul_rn((double)(ng - 8 + k), h);
    ya[k] = yb[k];
  }
  double y0 = neville8_exact(xa, ya, __dsub_rn(xa[7], delta));
  double y2 = neville8_exact(xa, ya, __dadd_rn(xa[7], delta));
  double y1 = yb[7];
  double y1p = __ddiv_rn(__dsub_rn(y2, y0), __dmul_rn(2.0, delta));
  double y1pp = __ddiv_rn(__dsub_rn(__dadd_rn(y2, y0), __dmul_rn(2.0, y1)), __dmul_rn(delta, delta));
  double r_max = __dadd_rn(__dmul_rn((double)(ng - 1), h), tail);
  double xx = __dsub_rn(r, r_max);
  double dx = -tail;
  double dx1 = __dmul_rn(y1p, dx);
  double dx2 = __dmul_rn(__dmul_rn(y1pp, dx), dx);
  double dd = __dadd_rn(__dsub_rn(__dmul_rn(10.0, y1), __dmul_rn(4.0, dx1)), __dmul_rn(0.5, dx2));
  double ee = __dsub_rn(__dadd_rn(__dmul_rn(-15.0, y1), __dmul_rn(7.0, dx1)), __dmul_rn(1.0, dx2));
  double ff = __dadd_rn(__dsub_rn(__dmul_rn(6.0, y1), __dmul_rn(3.0, dx1)), __dmul_rn(0.5, dx2));
  double xr = __ddiv_rn(xx, dx);
  double v = __dadd_rn(__dmul_rn(ff, xr), ee);
  v = __dadd_rn(__dmul_rn(v, xr), dd);
  v = __dmul_rn(__dmul_rn(__dmul_rn(v, xr), xr), xr);
  return v;
}

// Tail value for one table row.
__device__ double tail_value(const double* row, int ng, double h, double r) {
  return tail_value8(row + (ng - 9), ng, h, r);
}

// Lagrange weights of the 8-point window; the result is sum_k w[k] * table[last - 9 + k].
// Returns 0 for the polynomial region, 1 for the tail, 2 beyond it.
__device__ __forceinline__ int spline_weights(double r, double h, int ng, double* w, int& last) {
  const double q = r / h;
  const double fl = floor(q);
  if (!(fl < (double)ng)) {
    const double max_ind = (double)(ng - 1) + (double)(int)(1.0 / h);
    return (fl <= max_ind) ? 1 : 2;
  }
  int ind = (int)fl;
  last = ind + 5;
  if (last > ng) last = ng;
  if (last < 9) last = 9;
  const double t = q - (double)(last - 8);  // position in units of h from the first node
  double pre[8], suf[8];
  pre[0] = 1.0;
#pragma unroll
  for (int k = 0; k < 7; ++k) pre[k + 1] = pre[k] * (t - (double)k);
  suf[7] = 1.0;
#pragma unroll
  for (int k = 7; k > 0; --k) suf[k - 1] = suf[k] * (t - (double)k);
  // (-1)^(7-k) / (k! (7-k)!)
  const double cw[8] = {-1.0 / 5040.0, 1.0 / 720.0, -1.0 / 240.0, 1.0 / 144.0,
                        -1.0 / 144.0,  1.0 / 240.0, -1.0 / 720.0, 1.0 / 5040.0};
#pragma unroll
  for (int k = 0; k < 8; ++k) w[k] = pre[k] * suf[k] * cw[k];
  return 0;
}


// D^1 (3x3), D^2 (5x5), D^3 (7x7) of a rotation taking z to the unit bond
// direction u, into warp-private shared memory (lanes cooperate).
__device__ __forceinline__ void build_rotations(int lmax, double ux, double uy, double uz, double* D1, double* D2,
                                                double* D3, int lane) {
    // Frame: e1 perpendicular to u along the axis least aligned with u, e2 = u x e1.
  if (lmax >= 1) {
      const double ax = fabs(ux), ay = fabs(uy), az = fabs(uz);
      double e1x, e1y, e1z;
      if (ax <= ay && ax <= az) {        // a = x: e1 = x cross u
        e1x = 0.0; e1y = -uz; e1z = uy;
      } else if (ay <= az) {             // a = y
        e1x = uz; e1y = 0.0; e1z = -ux;
      } else {                           // a = z
        e1x = -uy; e1y = ux; e1z = 0.0;
      }
      const double inv = 1.0 / sqrt(e1x * e1x + e1y * e1y + e1z * e1z);
      e1x *= inv; e1y *= inv; e1z *= inv;
      const double e2x = uy * e1z - uz * e1y, e2y = uz * e1x - ux * e1z, e2z = ux * e1y - uy * e1x;
      // D^1[a][m] = R[c(a)][c(m)], R columns (e1, e2, u), c: -1 -> y, 0 -> z, 1 -> x
      if (lane < 9) {
        const int a = lane / 3, m = lane % 3;
        const int ca = (a == 0) ? 1 : (a == 1 ? 2 : 0);
        const int cm = (m == 0) ? 1 : (m == 1 ? 2 : 0);
        const double col0 = (ca == 0) ? e1x : (ca == 1 ? e1y : e1z);
        const double col1 = (ca == 0) ? e2x : (ca == 1 ? e2y : e2z);
        const double col2 = (ca == 0) ? ux : (ca == 1 ? uy : uz);
        D1[lane] = (cm == 0) ? col0 : (cm == 1 ? col1 : col2);
      }
      __syncwarp();
      if (lmax >= 2) {
        if (lane < 25) D2[lane] = rot_entry(2, lane, D1, D1);
        __syncwarp();
      }
      if (lmax >= 3) {
        for (int e = lane; e < 49; e += 32) D3[e] = rot_entry(3, e, D1, D2);
        __syncwarp();
      }
    }

}

}  // namespace
