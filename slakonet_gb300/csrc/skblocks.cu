// Real-space Slater-Koster blocks: spline lookup of the integrals and their
// rotation into the crystal frame, one warp per bond.
//
// Integrals.  The reference interpolates each table with an 8-point Neville
// scheme on the window ending n_interp_r = 4 points past floor(r/h)
// (slakonet/interpolation.py:107-170, 255-311).  Neville and Lagrange forms
// of that polynomial are the same function of r, and the Lagrange form is
// linear in the table values with weights that depend only on r and the
// grid, so one weight set per (bond, grid) serves every integral of the bond
// (and is exactly the pull-back the adjoint needs).  Beyond the last grid
// point the reference switches to a 5th-order tail whose second derivative
// is a finite difference over 1e-5 Bohr; that difference amplifies rounding
// by ~1e10, so the tail path re-evaluates the reference's Neville recursion
// with the same uncontracted operations (slakonet/interpolation.py:173-252).
//
// Rotation.  The block of a shell pair (la <= lb) is
//   B[a][b] = sum_{|m| <= la} V_|m|(d) D^la[a][m] D^lb[b][m],
// with D^l the rotation of the real spherical harmonics (m = -l..l: p as
// y, z, x; d as xy, yz, z2, xz, x2-y2) for any rotation taking the z axis to
// the bond direction u.  The reference evaluates closed-form tables for
// two such rotations (slakonet/slaterkoster.py:1013-1606); here D^1 comes
// from an orthonormal frame around u and D^2, D^3 from the Ivanic-Ruedenberg
// recursion (coefficients in rot_coeffs.cuh).
//
// Which table and orientation.  For bond (i, j, T) and shells (a on i, b on
// j): if la < lb, or la == lb and i <= j, the block comes from table
// (Zi, Zj, la, lb); otherwise from (Zj, Zi, lb, la) times (-1)^(la+lb).
// This is the real-space form of the reference's upper-triangle assembly
// with conjugate fill (slakonet/slaterkoster.py:204-405).
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

// Tail value for one table row (slakonet/interpolation.py:173-236, 241-252).
__device__ double tail_value(const double* row, int ng, double h, double r) {
  const double tail = 1.0, delta = 1e-5;
  double xa[8], ya[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    xa[k] = __dmul_rn((double)(ng - 8 + k), h);
    ya[k] = row[ng - 9 + k];
  }
  double y0 = neville8_exact(xa, ya, __dsub_rn(xa[7], delta));
  double y2 = neville8_exact(xa, ya, __dadd_rn(xa[7], delta));
  double y1 = row[ng - 2];
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

__global__ void __launch_bounds__(256) k_sk_blocks(
    int64_t n_bonds, const int32_t* __restrict__ bond_i, const int32_t* __restrict__ bond_j,
    const double* __restrict__ bond_d, const double* __restrict__ bond_u, const int64_t* __restrict__ bond_blk,
    const int32_t* __restrict__ atom_species, int nsp, const int32_t* __restrict__ sp_nshell,
    const int32_t* __restrict__ sp_shell_l, const int32_t* __restrict__ sp_norb,
    const int32_t* __restrict__ tab_index, const int64_t* __restrict__ tab_off,
    const int32_t* __restrict__ tab_ngrid, const double* __restrict__ tab_step,
    const double* __restrict__ tab_H, const double* __restrict__ tab_S, double* __restrict__ blk_H,
    double* __restrict__ blk_S, int32_t* __restrict__ status) {
  extern __shared__ double smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  double* my = smem + wib * WARP_SMEM;
  double* D0 = my;
  double* D1 = my + 1;
  double* D2 = my + 10;
  double* D3 = my + 35;
  double* VH = my + 84;
  double* VS = my + 116;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  if (lane == 0) D0[0] = 1.0;
  for (int64_t b = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib; b < n_bonds; b += nwarps) {
    const int gi = bond_i[b], gj = bond_j[b];
    const double d = bond_d[b];
    const double ux = bond_u[3 * b], uy = bond_u[3 * b + 1], uz = bond_u[3 * b + 2];
    const int spi = atom_species[gi], spj = atom_species[gj];
    const int nsi = sp_nshell[spi], nsj = sp_nshell[spj];
    int lmax = 0;
    for (int s = 0; s < nsi; ++s) lmax = max(lmax, sp_shell_l[4 * spi + s]);
    for (int s = 0; s < nsj; ++s) lmax = max(lmax, sp_shell_l[4 * spj + s]);

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

    // Integrals: items (sa, sb, beta).
    int n_items = 0;
    for (int sa = 0; sa < nsi; ++sa)
      for (int sb = 0; sb < nsj; ++sb)
        n_items += min(sp_shell_l[4 * spi + sa], sp_shell_l[4 * spj + sb]) + 1;
    for (int it = lane; it < n_items; it += 32) {
      int rem = it, sa = 0, sb = 0, la = 0, lb = 0, beta = 0;
      for (int p = 0; p < nsi * nsj; ++p) {
        const int a_ = p / nsj, b_ = p % nsj;
        const int l1 = sp_shell_l[4 * spi + a_], l2 = sp_shell_l[4 * spj + b_];
        const int cnt = min(l1, l2) + 1;
        if (rem < cnt) { sa = a_; sb = b_; la = l1; lb = l2; beta = rem; break; }
        rem -= cnt;
      }
      (void)sa; (void)sb;
      const bool direct = (la < lb) || (la == lb && gi <= gj);
      int t;
      double sign = 1.0;
      if (direct) {
        t = tab_index[((spi * nsp + spj) * 4 + la) * 4 + lb];
      } else {
        t = tab_index[((spj * nsp + spi) * 4 + lb) * 4 + la];
        if ((la + lb) & 1) sign = -1.0;
      }
      double vh = 0.0, vs = 0.0;
      if (t < 0) {
        atomicExch(status, SKN_ERR_ARG);
      } else {
        const int ng = tab_ngrid[t];
        const double h = tab_step[t];
        const double* rh = tab_H + tab_off[t] + (int64_t)beta * ng;
        const double* rs = tab_S + tab_off[t] + (int64_t)beta * ng;
        double w[8];
        int last = 0;
        const int region = spline_weights(d, h, ng, w, last);
        if (region == 0) {
          const double* yh = rh + (last - 9);
          const double* ys = rs + (last - 9);
#pragma unroll
          for (int k = 0; k < 8; ++k) {
            vh = fma(w[k], yh[k], vh);
            vs = fma(w[k], ys[k], vs);
          }
        } else if (region == 1) {
          vh = tail_value(rh, ng, h, d);
          vs = tail_value(rs, ng, h, d);
        }
      }
      VH[it] = sign * vh;
      VS[it] = sign * vs;
    }
    __syncwarp();

    // Assemble the column-major ni x nj block.
    const int ni = sp_norb[spi], nj = sp_norb[spj];
    const int64_t off = bond_blk[b];
    for (int e = lane; e < ni * nj; e += 32) {
      const int ar = e % ni, bc = e / ni;
      int sa = 0, oa = 0, la = 0;
      for (int s = 0; s < nsi; ++s) {
        const int l = sp_shell_l[4 * spi + s];
        if (ar < oa + 2 * l + 1) { sa = s; la = l; break; }
        oa += 2 * l + 1;
      }
      int sb = 0, ob = 0, lb = 0;
      for (int s = 0; s < nsj; ++s) {
        const int l = sp_shell_l[4 * spj + s];
        if (bc < ob + 2 * l + 1) { sb = s; lb = l; break; }
        ob += 2 * l + 1;
      }
      int base = 0;
      for (int p = 0; p < sa * nsj + sb; ++p) {
        const int a_ = p / nsj, b_ = p % nsj;
        base += min(sp_shell_l[4 * spi + a_], sp_shell_l[4 * spj + b_]) + 1;
      }
      const int am = ar - oa - la, bm = bc - ob - lb;  // -l..l
      const double* Da = (la == 0) ? D0 : (la == 1 ? D1 : (la == 2 ? D2 : D3));
      const double* Db = (lb == 0) ? D0 : (lb == 1 ? D1 : (lb == 2 ? D2 : D3));
      const int lo = min(la, lb);
      double hv = 0.0, sv = 0.0;
      for (int m = -lo; m <= lo; ++m) {
        const double p = rot_get(Da, la, am, m) * rot_get(Db, lb, bm, m);
        const int bo = m < 0 ? -m : m;
        hv = fma(VH[base + bo], p, hv);
        sv = fma(VS[base + bo], p, sv);
      }
      blk_H[off + e] = hv;
      blk_S[off + e] = sv;
    }
    __syncwarp();
  }
}

}  // namespace

extern "C" int skn_sk_blocks(int64_t n_bonds, const int32_t* bond_i, const int32_t* bond_j,
                             const double* bond_d, const double* bond_u, const int64_t* bond_blk,
                             const int32_t* atom_species, int n_species, const int32_t* sp_nshell,
                             const int32_t* sp_shell_l, const int32_t* sp_norb, const int32_t* tab_index,
                             const int64_t* tab_off, const int32_t* tab_ngrid, const double* tab_step,
                             const double* tab_H, const double* tab_S, double* blk_H, double* blk_S,
                             int32_t* status, cudaStream_t stream) {
  if (n_bonds < 0 || n_species <= 0) return SKN_ERR_ARG;
  if (n_bonds == 0) return SKN_OK;
  if (!bond_i || !bond_j || !bond_d || !bond_u || !bond_blk || !atom_species || !sp_nshell || !sp_shell_l ||
      !sp_norb || !tab_index || !tab_off || !tab_ngrid || !tab_step || !tab_H || !tab_S || !blk_H || !blk_S ||
      !status)
    return SKN_ERR_ARG;
  const int threads = 256;
  int64_t blocks = (n_bonds + 7) / 8;
  if (blocks > 152 * 16) blocks = 152 * 16;
  const size_t smem = (size_t)(threads / 32) * WARP_SMEM * sizeof(double);
  k_sk_blocks<<<(unsigned)blocks, threads, smem, stream>>>(
      n_bonds, bond_i, bond_j, bond_d, bond_u, bond_blk, atom_species, n_species, sp_nshell, sp_shell_l, sp_norb,
      tab_index, tab_off, tab_ngrid, tab_step, tab_H, tab_S, blk_H, blk_S, status);
  return cudaPeekAtLastError() == cudaSuccess ? SKN_OK : SKN_ERR_CUDA;
}
