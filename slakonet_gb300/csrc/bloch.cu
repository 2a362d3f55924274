// Bloch sums: H(k) = onsite + sum_T H(T) exp(i 2 pi k.T), and S(k) alike.
//
// CTAs stride over (structure, k) problems (blockIdx.x) and, for batches with
// fewer problems than the GPU has CTA slots, split each problem's atom pairs
// (blockIdx.y); each warp takes ordered atom pairs
// (i, j) and its lanes take the elements of the norb_i x norb_j block, so a
// warp walks one bond list with uniform trip count: every lane reads the same
// bond index and phase (broadcast) and its own block element (contiguous).
// The reference builds the same sums with a phase multiply and scatter_add
// over images followed by index scatters into [n, n, nk]
// (slakonet/slaterkoster.py:327-439, 971-1010); here every element is
// written once, k-major, column-major per k.
#include "skn_common.cuh"

namespace {

__global__ void __launch_bounds__(256) k_bloch(
    int n_prob, const int32_t* __restrict__ prob_struct, const int32_t* __restrict__ prob_k,
    const int64_t* __restrict__ hs_off, const int32_t* __restrict__ atom_ptr, const int32_t* __restrict__ orb_ptr,
    const int32_t* __restrict__ atom_orb_off, const int32_t* __restrict__ atom_norb,
    const int64_t* __restrict__ pair_base, const int64_t* __restrict__ pair_ptr,
    const int32_t* __restrict__ bond_img, const int64_t* __restrict__ bond_blk, const double* __restrict__ blk_H,
    const double* __restrict__ blk_S, const int32_t* __restrict__ image_range,
    const int64_t* __restrict__ phase_base, const double2* __restrict__ phases,
    const double* __restrict__ onsite_H, double2* __restrict__ H, double2* __restrict__ S) {
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int p = blockIdx.x; p < n_prob; p += gridDim.x) {
    const int s = prob_struct[p], k = prob_k[p];
    const int a0 = atom_ptr[s], N = atom_ptr[s + 1] - a0;
    const int o0 = orb_ptr[s], n = orb_ptr[s + 1] - o0;
    const int nimg = (2 * image_range[3 * s] + 1) * (2 * image_range[3 * s + 1] + 1) * (2 * image_range[3 * s + 2] + 1);
    const double2* ph = phases + phase_base[s] + (int64_t)k * nimg;
    double2* Hp = H + hs_off[p];
    double2* Sp = S + hs_off[p];
    const int64_t pb = pair_base[s];
    for (int q = blockIdx.y * nw + wib; q < N * N; q += nw * gridDim.y) {
      const int ib = q / N, ia = q % N;  // consecutive warps: consecutive row blocks of one column block
      const int gi = a0 + ia, gj = a0 + ib;
      const int ni = atom_norb[gi], nj = atom_norb[gj];
      const int oi = atom_orb_off[gi], oj = atom_orb_off[gj];
      const int64_t t0 = pair_ptr[pb + (int64_t)ia * N + ib], t1 = pair_ptr[pb + (int64_t)ia * N + ib + 1];
      for (int e = lane; e < ni * nj; e += 32) {
        const int al = e % ni, bl = e / ni;
        double2 h = make_double2(0.0, 0.0), sv = make_double2(0.0, 0.0);
        for (int64_t t = t0; t < t1; ++t) {
          const double2 f = ph[bond_img[t]];
          const int64_t o = bond_blk[t] + e;
          const double bh = blk_H[o], bs = blk_S[o];
          h.x = fma(bh, f.x, h.x);
          h.y = fma(bh, f.y, h.y);
          sv.x = fma(bs, f.x, sv.x);
          sv.y = fma(bs, f.y, sv.y);
        }
        if (ia == ib && al == bl) {
          h.x += onsite_H[o0 + oi + al];
          sv.x += 1.0;
        }
        const int64_t dst = (int64_t)(oj + bl) * n + (oi + al);
        Hp[dst] = h;
        Sp[dst] = sv;
      }
    }
  }
}

// The same sums organised by atom pair: a warp takes one ordered atom pair (i, j) of a structure and a
// chunk of up to BK of its k-points, and its lanes take (k-point, block element) items, k-point slowest,
// so warps stay full when blocks are small (1x1, 1x4, 4x4 orbitals) and no warp is left with a small
// cell's hundreds of k-points; every lane walks the pair's one bond list (bond indices and offsets are
// broadcast loads, block values contiguous per k-point).  Work units (pair, k-chunk) are numbered
// structure by structure: structure s owns N_s^2 * ceil(nk_s / BK) units from unit_base[s].  With
// `lower` only the blocks on or below the diagonal are formed (pairs with i >= j, and in diagonal blocks
// the entries on or below the diagonal): the eigensolvers read nothing else.  Each element is summed
// over the same bonds in the same order as k_bloch, so the values are bitwise the same.
constexpr int BK = 16;   // k-points per work unit

__global__ void __launch_bounds__(256) k_bloch_pairs(
    int n_struct, int64_t n_units, const int64_t* __restrict__ unit_base, const int32_t* __restrict__ k_ptr,
    const int64_t* __restrict__ hs_off, const int32_t* __restrict__ atom_ptr, const int32_t* __restrict__ orb_ptr,
    const int32_t* __restrict__ atom_orb_off, const int32_t* __restrict__ atom_norb,
    const int64_t* __restrict__ pair_base, const int64_t* __restrict__ pair_ptr,
    const int32_t* __restrict__ bond_img, const int64_t* __restrict__ bond_blk, const double* __restrict__ blk_H,
    const double* __restrict__ blk_S, const int32_t* __restrict__ image_range,
    const int64_t* __restrict__ phase_base, const double2* __restrict__ phases,
    const double* __restrict__ onsite_H, int lower, double2* __restrict__ H, double2* __restrict__ S) {
  const int lane = threadIdx.x & 31;
  const int64_t wstride = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t u = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); u < n_units; u += wstride) {
    int lo = 0, hi = n_struct - 1;                  // the structure: last s with unit_base[s] <= u
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (unit_base[mid] <= u) lo = mid; else hi = mid - 1;
    }
    const int s = lo;
    const int p0 = k_ptr[s], nk = k_ptr[s + 1] - p0;
    const int nkc = (nk + BK - 1) / BK;
    const int64_t local = u - unit_base[s];
    const int q = (int)(local / nkc), kc = (int)(local % nkc);
    const int a0 = atom_ptr[s], N = atom_ptr[s + 1] - a0;
    const int ib = q / N, ia = q % N;               // consecutive units: k-chunks, then row blocks
    if (lower && ia < ib) continue;
    const int gi = a0 + ia, gj = a0 + ib;
    const int ni = atom_norb[gi], nj = atom_norb[gj];
    const int oi = atom_orb_off[gi], oj = atom_orb_off[gj];
    const int o0 = orb_ptr[s], n = orb_ptr[s + 1] - o0;
    const int k0 = kc * BK, kcnt = min(BK, nk - k0);
    const int nimg = (2 * image_range[3 * s] + 1) * (2 * image_range[3 * s + 1] + 1) * (2 * image_range[3 * s + 2] + 1);
    const double2* ph = phases + phase_base[s];
    const int64_t pq = pair_base[s] + (int64_t)ia * N + ib;     // bonds of (i, j): row-major pair index
    const int64_t t0 = pair_ptr[pq], t1 = pair_ptr[pq + 1];
    const int ne = ni * nj;
    const bool diag = ia == ib;
    for (int it = lane; it < kcnt * ne; it += 32) {
      const int k = k0 + it / ne, e = it % ne;
      const int al = e % ni, bl = e / ni;
      if (lower && diag && al < bl) continue;
      const double2* phk = ph + (int64_t)k * nimg;
      double2 h = make_double2(0.0, 0.0), sv = make_double2(0.0, 0.0);
      for (int64_t t = t0; t < t1; ++t) {
        const double2 f = phk[bond_img[t]];
        const int64_t o = bond_blk[t] + e;
        const double bh = blk_H[o], bs = blk_S[o];
        h.x = fma(bh, f.x, h.x);
        h.y = fma(bh, f.y, h.y);
        sv.x = fma(bs, f.x, sv.x);
        sv.y = fma(bs, f.y, sv.y);
      }
      if (diag && al == bl) {
        h.x += onsite_H[o0 + oi + al];
        sv.x += 1.0;
      }
      const int64_t dst = hs_off[p0 + k] + (int64_t)(oj + bl) * n + (oi + al);
      H[dst] = h;
      S[dst] = sv;
    }
  }
}

}  // namespace

extern "C" int skn_bloch_pairs(int n_struct, int64_t n_units, const int64_t* unit_base, const int32_t* k_ptr,
                               const int64_t* hs_off, const int32_t* atom_ptr, const int32_t* orb_ptr,
                               const int32_t* atom_orb_off, const int32_t* atom_norb, const int64_t* pair_base,
                               const int64_t* pair_ptr, const int32_t* bond_img, const int64_t* bond_blk,
                               const double* blk_H, const double* blk_S, const int32_t* image_range,
                               const int64_t* phase_base, const double* phases, const double* onsite_H, int lower,
                               double* H, double* S, cudaStream_t stream) {
  if (n_struct < 0 || n_units < 0) return SKN_ERR_ARG;
  if (n_struct == 0 || n_units == 0) return SKN_OK;
  if (!unit_base || !k_ptr || !hs_off || !atom_ptr || !orb_ptr || !atom_orb_off || !atom_norb || !pair_base ||
      !pair_ptr || !image_range || !phase_base || !phases || !onsite_H || !H || !S)
    return SKN_ERR_ARG;
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bloch_pairs, 256, 0) != cudaSuccess || per_sm < 1)
    per_sm = 1;
  const int64_t slots = (int64_t)per_sm * (sms > 0 ? sms : 1);   // one wave of resident CTAs, warps stride over units
  const int64_t need = (n_units + 7) / 8;
  const unsigned grid = (unsigned)(need < slots ? need : slots);
  k_bloch_pairs<<<grid, 256, 0, stream>>>(n_struct, n_units, unit_base, k_ptr, hs_off, atom_ptr, orb_ptr,
                                          atom_orb_off, atom_norb, pair_base, pair_ptr, bond_img, bond_blk, blk_H,
                                          blk_S, image_range, phase_base, (const double2*)phases, onsite_H, lower,
                                          (double2*)H, (double2*)S);
  return cudaPeekAtLastError() == cudaSuccess ? SKN_OK : SKN_ERR_CUDA;
}

extern "C" int skn_bloch(int n_prob, const int32_t* prob_struct, const int32_t* prob_k, const int64_t* hs_off,
                         const int32_t* atom_ptr, const int32_t* orb_ptr, const int32_t* orb_atom,
                         const int32_t* atom_orb_off, const int32_t* atom_norb, const int64_t* pair_base,
                         const int64_t* pair_ptr, const int32_t* bond_img, const int64_t* bond_blk,
                         const double* blk_H, const double* blk_S, const int32_t* image_range,
                         const int64_t* phase_base, const double* phases, const double* onsite_H,
                         int max_n, double* H, double* S, cudaStream_t stream) {
  (void)orb_atom;
  if (n_prob < 0) return SKN_ERR_ARG;
  if (n_prob == 0) return SKN_OK;
  if (!prob_struct || !prob_k || !hs_off || !atom_ptr || !orb_ptr || !atom_orb_off || !atom_norb || !pair_base ||
      !pair_ptr || !image_range || !phase_base || !phases || !onsite_H || !H || !S)
    return SKN_ERR_ARG;
  if (max_n < 0) return SKN_ERR_ARG;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int slots = 8 * (sms > 0 ? sms : 1);          // 256-thread CTAs resident at once
  const int bx = n_prob < slots ? n_prob : slots;
  // split problems over blockIdx.y only as far as there are warps of atom pairs to give out
  const int64_t pair_warps = ((int64_t)max_n * max_n + 7) / 8;
  int64_t by = (slots + bx - 1) / bx;
  if (by > pair_warps) by = pair_warps;
  if (by < 1) by = 1;
  if (by > 65535) by = 65535;
  k_bloch<<<dim3(bx, (unsigned)by), 256, 0, stream>>>(n_prob, prob_struct, prob_k, hs_off, atom_ptr, orb_ptr, atom_orb_off, atom_norb,
                                      pair_base, pair_ptr, bond_img, bond_blk, blk_H, blk_S, image_range, phase_base,
                                      (const double2*)phases, onsite_H, (double2*)H, (double2*)S);
  return cudaPeekAtLastError() == cudaSuccess ? SKN_OK : SKN_ERR_CUDA;
}
