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
#include "sk_common.cuh"

namespace {

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

    build_rotations(lmax, ux, uy, uz, D1, D2, D3, lane);

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
