// Hand-written adjoint of the eigenvalues with respect to the SK tables.
//
// For a loss L(e) with g = dL/de, first-order perturbation theory of
// H c = e S c (c^H S c = 1) gives de_n = c_n^H (dH - e_n dS) c_n, so
//   dL/dH(k)_ab =  G_ab = sum_n g_n conj(c_n[a]) c_n[b],
//   dL/dS(k)_ab = -F_ab, F_ab = sum_n g_n e_n conj(c_n[a]) c_n[b].
// H(k)_ab = sum over bonds (i -> j + T) of the real block B_ab(T) exp(i 2 pi k.T),
// so dL/dB_ab(T) = sum_k Re(G_ab(k) exp(i 2 pi k.T)) (and -F for S).
// The block is B = sign sum_m V_|m|(d) D^la[a][m] D^lb[b][m] and V is a
// fixed linear combination (Lagrange weights, or the tail functional) of
// eight table entries, so the pull-back onto the tables is a weighted
// scatter-add.  H(k) and S(k) are not stored: G and F come from the
// eigenvectors, the blocks' geometry is recomputed per bond.
//
// The reference differentiates with autograd through torch.linalg.eigh,
// whose backward (slakonet/utils.py:387-473) drops the complex conjugate for
// Hermitian inputs; the gradients here follow the formula above and are
// checked against central finite differences and against the reference's
// autograd with the conjugate restored.
#include "sk_common.cuh"

namespace {

constexpr double H2E = 27.211;

// G, F per problem, 16x16 output tiles staged through shared memory.
__global__ void __launch_bounds__(256) k_adj_projectors(int n_prob, const int32_t* __restrict__ nvec,
                                                        const int64_t* __restrict__ hs_off,
                                                        const int64_t* __restrict__ eig_off,
                                                        const double2* __restrict__ C, const double* __restrict__ eig,
                                                        const double* __restrict__ g, const int32_t* __restrict__ status,
                                                        double2* __restrict__ G, double2* __restrict__ F) {
  __shared__ double2 ca[16][17], cb[16][17];
  __shared__ double gj[16], gej[16];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  for (int p = blockIdx.x; p < n_prob; p += gridDim.x) {
    const int n = nvec[p];
    const double2* Cp = C + hs_off[p];
    const double* ep = eig + eig_off[p];
    const double* gp = g + eig_off[p];
    double2* Gp = G + hs_off[p];
    double2* Fp = F + hs_off[p];
    if (status != nullptr && status[p] != SKN_OK) {   // failed problem: NaN vectors carry no gradient
      for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        Gp[e] = make_double2(0.0, 0.0);
        Fp[e] = make_double2(0.0, 0.0);
      }
      continue;
    }
    for (int a0 = 0; a0 < n; a0 += 16) {
      for (int b0 = 0; b0 < n; b0 += 16) {
        const int a = a0 + tx, b = b0 + ty;
        double2 accG = make_double2(0.0, 0.0), accF = make_double2(0.0, 0.0);
        for (int j0 = 0; j0 < n; j0 += 16) {
          const int jc = j0 + tx;
          ca[ty][tx] = (a0 + ty < n && jc < n) ? Cp[(int64_t)(a0 + ty) * n + jc] : make_double2(0.0, 0.0);
          cb[ty][tx] = (b0 + ty < n && jc < n) ? Cp[(int64_t)(b0 + ty) * n + jc] : make_double2(0.0, 0.0);
          if (threadIdx.x < 16) {
            const int j = j0 + threadIdx.x;
            gj[threadIdx.x] = j < n ? gp[j] : 0.0;
            gej[threadIdx.x] = j < n ? gp[j] * ep[j] : 0.0;
          }
          __syncthreads();
#pragma unroll 4
          for (int c = 0; c < 16; ++c) {
            const double2 x = ca[tx][c], y = cb[ty][c];
            // conj(x) * y
            const double pr = fma(x.x, y.x, x.y * y.y);
            const double pi = fma(x.x, y.y, -x.y * y.x);
            accG.x = fma(gj[c], pr, accG.x);
            accG.y = fma(gj[c], pi, accG.y);
            accF.x = fma(gej[c], pr, accF.x);
            accF.y = fma(gej[c], pi, accF.y);
          }
          __syncthreads();
        }
        if (a < n && b < n) {
          Gp[(int64_t)b * n + a] = accG;
          Fp[(int64_t)b * n + a] = accF;
        }
      }
    }
  }
}

// dL/dB per bond and block element: sum over the structure's k-points.
__global__ void __launch_bounds__(256) k_adj_bloch(
    int64_t n_bonds, const int32_t* __restrict__ bond_i, const int32_t* __restrict__ bond_j,
    const int32_t* __restrict__ bond_img, const int64_t* __restrict__ bond_blk,
    const int32_t* __restrict__ atom_struct, const int32_t* __restrict__ atom_orb_off,
    const int32_t* __restrict__ atom_norb, const int32_t* __restrict__ struct_prob0, const int32_t* __restrict__ nkv,
    const int32_t* __restrict__ nbv, const int64_t* __restrict__ hs_off, const int32_t* __restrict__ image_range,
    const int64_t* __restrict__ phase_base, const double2* __restrict__ phases, const double2* __restrict__ G,
    const double2* __restrict__ F, double* __restrict__ gH, double* __restrict__ gS) {
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t t = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); t < n_bonds; t += nwarps) {
    const int gi = bond_i[t], gj = bond_j[t];
    const int s = atom_struct[gi];
    const int ni = atom_norb[gi], nj = atom_norb[gj];
    const int oi = atom_orb_off[gi], oj = atom_orb_off[gj];
    const int nk = nkv[s], n = nbv[s], p0 = struct_prob0[s];
    const int nimg = (2 * image_range[3 * s] + 1) * (2 * image_range[3 * s + 1] + 1) * (2 * image_range[3 * s + 2] + 1);
    const double2* ph = phases + phase_base[s] + bond_img[t];
    const int64_t blk = bond_blk[t];
    for (int e = lane; e < ni * nj; e += 32) {
      const int a = oi + e % ni, b = oj + e / ni;
      double ah = 0.0, as = 0.0;
      for (int k = 0; k < nk; ++k) {
        const double2 f = ph[(int64_t)k * nimg];
        const int64_t o = hs_off[p0 + k] + (int64_t)b * n + a;
        const double2 gv = G[o], fv = F[o];
        ah = fma(gv.x, f.x, fma(-gv.y, f.y, ah));
        as = fma(-fv.x, f.x, fma(fv.y, f.y, as));
      }
      gH[blk + e] = ah;
      gS[blk + e] = as;
    }
  }
}

// Pull the block gradients back through the rotation and the spline onto the tables.
__global__ void __launch_bounds__(256) k_adj_tables(
    int64_t n_bonds, const int32_t* __restrict__ bond_i, const int32_t* __restrict__ bond_j,
    const double* __restrict__ bond_d, const double* __restrict__ bond_u, const int64_t* __restrict__ bond_blk,
    const int32_t* __restrict__ atom_species, int nsp, const int32_t* __restrict__ sp_nshell,
    const int32_t* __restrict__ sp_shell_l, const int32_t* __restrict__ sp_norb,
    const int32_t* __restrict__ tab_index, const int64_t* __restrict__ tab_off,
    const int32_t* __restrict__ tab_ngrid, const double* __restrict__ tab_step, const double* __restrict__ gH,
    const double* __restrict__ gS, double* __restrict__ dtab_H, double* __restrict__ dtab_S) {
  extern __shared__ double smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  double* my = smem + wib * WARP_SMEM;
  double* D0 = my;
  double* D1 = my + 1;
  double* D2 = my + 10;
  double* D3 = my + 35;
  const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
  if (lane == 0) D0[0] = 1.0;
  for (int64_t bnd = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib; bnd < n_bonds; bnd += nwarps) {
    const int gi = bond_i[bnd], gj = bond_j[bnd];
    const double d = bond_d[bnd];
    const int spi = atom_species[gi], spj = atom_species[gj];
    const int nsi = sp_nshell[spi], nsj = sp_nshell[spj];
    const int ni = sp_norb[spi];
    int lmax = 0;
    for (int s = 0; s < nsi; ++s) lmax = max(lmax, sp_shell_l[4 * spi + s]);
    for (int s = 0; s < nsj; ++s) lmax = max(lmax, sp_shell_l[4 * spj + s]);
    build_rotations(lmax, bond_u[3 * bnd], bond_u[3 * bnd + 1], bond_u[3 * bnd + 2], D1, D2, D3, lane);
    __syncwarp();
    const double* bh = gH + bond_blk[bnd];
    const double* bs = gS + bond_blk[bnd];
    int n_items = 0;
    for (int sa = 0; sa < nsi; ++sa)
      for (int sb = 0; sb < nsj; ++sb) n_items += min(sp_shell_l[4 * spi + sa], sp_shell_l[4 * spj + sb]) + 1;
    for (int it = lane; it < n_items; it += 32) {
      int rem = it, sa = 0, sb = 0, la = 0, lb = 0, beta = 0;
      for (int p = 0; p < nsi * nsj; ++p) {
        const int a_ = p / nsj, b_ = p % nsj;
        const int l1 = sp_shell_l[4 * spi + a_], l2 = sp_shell_l[4 * spj + b_];
        const int cnt = min(l1, l2) + 1;
        if (rem < cnt) { sa = a_; sb = b_; la = l1; lb = l2; beta = rem; break; }
        rem -= cnt;
      }
      int oa = 0, ob = 0;
      for (int q = 0; q < sa; ++q) oa += 2 * sp_shell_l[4 * spi + q] + 1;
      for (int q = 0; q < sb; ++q) ob += 2 * sp_shell_l[4 * spj + q] + 1;
      const bool direct = (la < lb) || (la == lb && gi <= gj);
      int t;
      double sign = 1.0;
      if (direct) {
        t = tab_index[((spi * nsp + spj) * 4 + la) * 4 + lb];
      } else {
        t = tab_index[((spj * nsp + spi) * 4 + lb) * 4 + la];
        if ((la + lb) & 1) sign = -1.0;
      }
      if (t < 0) continue;
      const double* Da = (la == 0) ? D0 : (la == 1 ? D1 : (la == 2 ? D2 : D3));
      const double* Db = (lb == 0) ? D0 : (lb == 1 ? D1 : (lb == 2 ? D2 : D3));
      double vh = 0.0, vs = 0.0;
      for (int am = -la; am <= la; ++am) {
        for (int bm = -lb; bm <= lb; ++bm) {
          double pr = rot_get(Da, la, am, beta) * rot_get(Db, lb, bm, beta);
          if (beta > 0) pr = fma(rot_get(Da, la, am, -beta), rot_get(Db, lb, bm, -beta), pr);
          const int64_t o = (int64_t)(ob + bm + lb) * ni + (oa + am + la);
          vh = fma(bh[o], pr, vh);
          vs = fma(bs[o], pr, vs);
        }
      }
      vh *= sign;
      vs *= sign;
      const int ng = tab_ngrid[t];
      const double h = tab_step[t];
      double* th = dtab_H + tab_off[t] + (int64_t)beta * ng;
      double* ts = dtab_S + tab_off[t] + (int64_t)beta * ng;
      double w[8];
      int last = 0;
      const int region = spline_weights(d, h, ng, w, last);
      if (region == 0) {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          atomicAdd(th + last - 9 + k, w[k] * vh);
          atomicAdd(ts + last - 9 + k, w[k] * vs);
        }
      } else if (region == 1) {
        for (int k = 0; k < 8; ++k) {
          double unit[8] = {0, 0, 0, 0, 0, 0, 0, 0};
          unit[k] = 1.0;
          const double c = tail_value8(unit, ng, h, d);
          atomicAdd(th + ng - 9 + k, c * vh);
          atomicAdd(ts + ng - 9 + k, c * vs);
        }
      }
    }
    __syncwarp();
  }
}

__device__ __forceinline__ double lin_grid(double lo, double hi, int n, int i) {
  if (n == 1) return lo;
  const double step = (hi - lo) / (double)(n - 1);
  return (i < n / 2) ? fma(step, (double)i, lo) : fma(-step, (double)(n - 1 - i), hi);
}

// dL/de from dL/dDOS (the DOS's dependence on each eigenvalue; mu is not
// differentiated, as in the reference where fermi_search detaches it).
__global__ void __launch_bounds__(256) k_dos_backward(const int64_t* __restrict__ eig_off,
                                                      const int32_t* __restrict__ nkv, const int32_t* __restrict__ nbv,
                                                      const int64_t* __restrict__ kw_off,
                                                      const double* __restrict__ kweights,
                                                      const double* __restrict__ eigall, const double* __restrict__ muv,
                                                      double e_lo, double e_hi, int npts, double sigma, double window,
                                                      const double* __restrict__ gdos, double* __restrict__ geig) {
  const int s = blockIdx.y;
  const int nk = nkv[s], nb = nbv[s];
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nk * nb) return;
  const double mu = muv[s];
  if (!(mu == mu)) return;
  const double x = (eigall[eig_off[s] + f] - mu) * H2E;
  const double wk = kweights[kw_off[s] + f / nb];
  const double inv_sigma = 1.0 / sigma;
  const double inv_norm = 1.0 / (sigma * sqrt(2.0 * 3.141592653589793));
  int i0 = 0, i1 = npts - 1;
  if (window > 0.0 && npts > 1) {
    const double step = (e_hi - e_lo) / (double)(npts - 1);
    i0 = max(0, (int)floor((x - window * sigma - e_lo) / step) - 1);
    i1 = min(npts - 1, (int)ceil((x + window * sigma - e_lo) / step) + 1);
  }
  const double* gd = gdos + (int64_t)s * npts;
  double acc = 0.0;
  for (int i = i0; i <= i1; ++i) {
    const double t = (lin_grid(e_lo, e_hi, npts, i) - x) * inv_sigma;
    acc = fma(gd[i], exp(-0.5 * (t * t)) * inv_norm * t * inv_sigma, acc);
  }
  geig[eig_off[s] + f] += wk * acc * H2E;
}

}  // namespace

extern "C" int skn_adj_projectors(int n_prob, const int32_t* n, const int64_t* hs_off, const int64_t* eig_off,
                                  const double* vec, const double* eig, const double* grad_eig,
                                  const int32_t* status, double* G, double* F, cudaStream_t stream) {
  if (n_prob < 0) return SKN_ERR_ARG;
  if (n_prob == 0) return SKN_OK;
  if (!n || !hs_off || !eig_off || !vec || !eig || !grad_eig || !G || !F) return SKN_ERR_ARG;
  const int grid = n_prob < 152 * 8 ? n_prob : 152 * 8;
  k_adj_projectors<<<grid, 256, 0, stream>>>(n_prob, n, hs_off, eig_off, (const double2*)vec, eig, grad_eig,
                                             status, (double2*)G, (double2*)F);
  return cudaPeekAtLastError() == cudaSuccess ? SKN_OK : SKN_ERR_CUDA;
}

extern "C" int skn_adj_bloch(int64_t n_bonds, const int32_t* bond_i, const int32_t* bond_j, const int32_t* bond_img,
                             const int64_t* bond_blk, const int32_t* atom_struct, const int32_t* atom_orb_off,
                             const int32_t* atom_norb, const int32_t* struct_prob0, const int32_t* nk,
                             const int32_t* nb, const int64_t* hs_off, const int32_t* image_range,
                             const int64_t* phase_base, const double* phases, const double* G, const double* F,
                             double* grad_blk_H, double* grad_blk_S, cudaStream_t stream) {
  if (n_bonds < 0) return SKN_ERR_ARG;
  if (n_bonds == 0) return SKN_OK;
  if (!bond_i || !bond_j || !bond_img || !bond_blk || !atom_struct || !atom_orb_off || !atom_norb || !struct_prob0 ||
      !nk || !nb || !hs_off || !image_range || !phase_base || !phases || !G || !F || !grad_blk_H || !grad_blk_S)
    return SKN_ERR_ARG;
  int64_t blocks = (n_bonds + 7) / 8;
  if (blocks > 152 * 16) blocks = 152 * 16;
  k_adj_bloch<<<(unsigned)blocks, 256, 0, stream>>>(n_bonds, bond_i, bond_j, bond_img, bond_blk, atom_struct,
                                                    atom_orb_off, atom_norb, struct_prob0, nk, nb, hs_off, image_range,
                                                    phase_base, (const double2*)phases, (const double2*)G,
                                                    (const double2*)F, grad_blk_H, grad_blk_S);
  return cudaPeekAtLastError() == cudaSuccess ? SKN_OK : SKN_ERR_CUDA;
}

extern "C" int skn_adj_tables(int64_t n_bonds, const int32_t* bond_i, const int32_t* bond_j, const double* bond_d,
                              const double* bond_u, const int64_t* bond_blk, const int32_t* atom_species,
                              int n_species, const int32_t* sp_nshell, const int32_t* sp_shell_l,
                              const int32_t* sp_norb, const int32_t* tab_index, const int64_t* tab_off,
                              const int32_t* tab_ngrid, const double* tab_step, const double* grad_blk_H,
                              const double* grad_blk_S, double* grad_tab_H, double* grad_tab_S, cudaStream_t stream) {
  if (n_bonds < 0 || n_species <= 0) return SKN_ERR_ARG;
  if (n_bonds == 0) return SKN_OK;
  if (!bond_i || !bond_j || !bond_d || !bond_u || !bond_blk || !atom_species || !sp_nshell || !sp_shell_l ||
      !sp_norb || !tab_index || !tab_off || !tab_ngrid || !tab_step || !grad_blk_H || !grad_blk_S || !grad_tab_H ||
      !grad_tab_S)
    return SKN_ERR_ARG;
  int64_t blocks = (n_bonds + 7) / 8;
  if (blocks > 152 * 16) blocks = 152 * 16;
  const size_t smem = 8 * WARP_SMEM * sizeof(double);
  k_adj_tables<<<(unsigned)blocks, 256, smem, stream>>>(n_bonds, bond_i, bond_j, bond_d, bond_u, bond_blk,
                                                        atom_species, n_species, sp_nshell, sp_shell_l, sp_norb,
                                                        tab_index, tab_off, tab_ngrid, tab_step, grad_blk_H,
                                                        grad_blk_S, grad_tab_H, grad_tab_S);
  return cudaPeekAtLastError() == cudaSuccess ? SKN_OK : SKN_ERR_CUDA;
}

extern "C" int skn_dos_backward(int n_struct, const int64_t* eig_off, const int32_t* nk, const int32_t* nb,
                                const int64_t* kw_off, const double* kweights, const double* eig, const double* mu,
                                double e_lo, double e_hi, int npts, double sigma, double window_sigmas,
                                const double* grad_dos, double* grad_eig, int max_count, cudaStream_t stream) {
  if (n_struct < 0 || npts <= 0 || !(sigma > 0.0) || window_sigmas < 0.0 || max_count < 0) return SKN_ERR_ARG;
  if (n_struct == 0 || max_count == 0) return SKN_OK;
  if (!eig_off || !nk || !nb || !kw_off || !kweights || !eig || !mu || !grad_dos || !grad_eig) return SKN_ERR_ARG;
  if (n_struct > 65535) return SKN_ERR_CAPACITY;
  dim3 g((max_count + 255) / 256, n_struct);
  k_dos_backward<<<g, 256, 0, stream>>>(eig_off, nk, nb, kw_off, kweights, eig, mu, e_lo, e_hi, npts, sigma,
                                        window_sigmas, grad_dos, grad_eig);
  return cudaPeekAtLastError() == cudaSuccess ? SKN_OK : SKN_ERR_CUDA;
}
