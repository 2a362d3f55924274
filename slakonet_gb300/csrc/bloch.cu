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
// cell's hundreds of k-points.  With `lower` only the blocks on or below the diagonal are formed (pairs
// with i >= j, and in diagonal blocks the entries on or below the diagonal): the eigensolvers read
// nothing else.
//
// Work units (pair, k-chunk) are numbered structure by structure from unit_base[s], column atom j
// slowest, then the k-chunk, then the row atom i fastest (i >= j with `lower`): structure s owns
// ceil(nk_s / BK) * N_s^2 units, or ceil(nk_s / BK) * N_s (N_s + 1) / 2 with `lower`.  The warps of a
// CTA take consecutive units, so they write the adjacent row blocks of one column block of the same
// k-points' matrices together: long runs of each column instead of one block's few rows in many
// matrices, which is what the write stream's DRAM efficiency depends on (the sums themselves are a
// small part of the work: most atom pairs of a large cell have no bond within the cutoff).
//
// Per unit the warp stages the pair's bonds in shared memory, BT at a time: each bond's block offset and
// its phase at every k-point of the chunk (one gather per bond and k-point instead of one per item and
// bond).  The item loop then reads offsets and phases from shared memory (broadcast: a warp's items span
// at most two k-points of a block) and the block values from global memory (contiguous in the element
// index, shared by the chunk's k-points through L1).  Item coordinates come from multiply-high division
// by the block sizes.  A pair with more than BT bonds takes several passes, each continuing the sums from
// the values the previous pass stored, so every element is summed over the same bonds in the same order
// as k_bloch: the values are bitwise the same.
//
// Units differ in size by two orders of magnitude (a 1x1 block at one k-point to 16x16 blocks at 8), so
// the grid holds one unit per warp and the hardware's block scheduler balances the SMs: a persistent grid
// striding over the units left 40% of the SM cycles idle in its tail (ncu, 16-structure sample).  Measured
// on GB300 over the 256-structure uneven batch (4.4 GB of lower triangles): 3.0 ms with the persistent
// grid and 16-k-point units, 1.97 ms with one unit per warp, 1.73 ms with 8-k-point units in 4-warp CTAs
// (8 per SM).  4-k-point units write faster without bonds but stage each pair's bonds twice as often.
constexpr int BK = 8;    // k-points per work unit
constexpr int BT = 16;   // bonds staged per pass
constexpr int BW = 4;    // warps per CTA

// floor(a / d) for a * d < 2^32 by a multiply-high with m = floor((2^32 - 1) / d) + 1 (d >= 2); d = 1 is
// the identity.
SKN_DEVINL uint32_t div_magic(uint32_t d) { return d <= 1u ? 0u : 0xFFFFFFFFu / d + 1u; }
SKN_DEVINL uint32_t div_by(uint32_t a, uint32_t d, uint32_t m) { return d <= 1u ? a : __umulhi(a, m); }

__global__ void __launch_bounds__(BW * 32, 8) k_bloch_pairs(
    int n_struct, int64_t n_units, const int64_t* __restrict__ unit_base, const int32_t* __restrict__ k_ptr,
    const int64_t* __restrict__ hs_off, const int32_t* __restrict__ atom_ptr, const int32_t* __restrict__ orb_ptr,
    const int32_t* __restrict__ atom_orb_off, const int32_t* __restrict__ atom_norb,
    const int64_t* __restrict__ pair_base, const int64_t* __restrict__ pair_ptr,
    const int32_t* __restrict__ bond_img, const int64_t* __restrict__ bond_blk, const double* __restrict__ blk_H,
    const double* __restrict__ blk_S, const int32_t* __restrict__ image_range,
    const int64_t* __restrict__ phase_base, const double2* __restrict__ phases,
    const double* __restrict__ onsite_H, int lower, double2* __restrict__ H, double2* __restrict__ S) {
  __shared__ double2 s_ph[BW][BK][BT];
  __shared__ int64_t s_off[BW][BT];
  __shared__ int64_t s_hs[BW][BK];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  {
    const int64_t u = (int64_t)blockIdx.x * BW + w;
    if (u >= n_units) return;
    int lo = 0, hi = n_struct - 1;                  // the structure: last s with unit_base[s] <= u
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (unit_base[mid] <= u) lo = mid; else hi = mid - 1;
    }
    const int s = lo;
    const int p0 = k_ptr[s];
    const int nk = k_ptr[s + 1] - p0;
    const int nkc = (nk + BK - 1) / BK;
    const int a0 = atom_ptr[s];
    const int N = atom_ptr[s + 1] - a0;
    const int o0 = orb_ptr[s];
    const int n = orb_ptr[s + 1] - o0;
    const int nimg =
        (2 * image_range[3 * s] + 1) * (2 * image_range[3 * s + 1] + 1) * (2 * image_range[3 * s + 2] + 1);
    const double2* ph = phases + phase_base[s];
    const int64_t pb = pair_base[s];
    const int64_t local = u - unit_base[s];
    int ib, ia, kc;
    if (lower) {
      // column atom j owns nkc (N - j) units from nkc (j N - j (j - 1) / 2): the largest such j
      const int64_t x = local / nkc;                // units of whole row-atom runs before this one
      const double b = 2.0 * N + 1.0;
      ib = (int)floor(0.5 * (b - sqrt(fmax(b * b - 8.0 * (double)x, 0.0))));
      ib = max(0, min(ib, N - 1));
      while (ib > 0 && (int64_t)ib * (2 * N - ib + 1) / 2 > x) --ib;
      while (ib + 1 < N && (int64_t)(ib + 1) * (2 * N - ib) / 2 <= x) ++ib;
      const int64_t rem = local - (int64_t)nkc * ((int64_t)ib * (2 * N - ib + 1) / 2);
      const int rows = N - ib;
      kc = (int)(rem / rows);
      ia = ib + (int)(rem - (int64_t)kc * rows);
    } else {
      const int64_t q = local / N;
      ia = (int)(local - q * N);
      kc = (int)(q % nkc);
      ib = (int)(q / nkc);
    }
    const int gi = a0 + ia, gj = a0 + ib;
    const int ni = atom_norb[gi], nj = atom_norb[gj];
    const int oi = atom_orb_off[gi], oj = atom_orb_off[gj];
    const int k0 = kc * BK, kcnt = min(BK, nk - k0);
    const int64_t pq = pb + (int64_t)ia * N + ib;   // bonds of (i, j): row-major pair index
    const int64_t t0 = pair_ptr[pq], t1 = pair_ptr[pq + 1];
    if (lane < kcnt) s_hs[w][lane] = hs_off[p0 + k0 + lane];
    const int ne = ni * nj, items = kcnt * ne;
    const uint32_t mne = div_magic((uint32_t)ne), mni = div_magic((uint32_t)ni);
    const bool diag = ia == ib;
    const double* onsite = onsite_H + o0 + oi;
    for (int64_t tb = t0;; tb += BT) {
      const int nbc = (int)min((int64_t)BT, t1 - tb);   // bonds of this pass (0 for a pair without bonds)
      __syncwarp();
      if (lane < nbc) {
        s_off[w][lane] = bond_blk[tb + lane];
        const int img = bond_img[tb + lane];
        for (int kl = 0; kl < kcnt; ++kl) s_ph[w][kl][lane] = ph[(int64_t)(k0 + kl) * nimg + img];
      }
      __syncwarp();
      const bool first = tb == t0, last = tb + BT >= t1;
      for (int it = lane; it < items; it += 32) {
        const int kl = (int)div_by((uint32_t)it, (uint32_t)ne, mne);
        const int e = it - kl * ne;
        const int bl = (int)div_by((uint32_t)e, (uint32_t)ni, mni);
        const int al = e - bl * ni;
        if (lower && diag && al < bl) continue;
        const int64_t dst = s_hs[w][kl] + (int64_t)(oj + bl) * n + (oi + al);
        double2 h = make_double2(0.0, 0.0), sv = make_double2(0.0, 0.0);
        if (!first) {
          h = H[dst];
          sv = S[dst];
        }
        const double2* phk = s_ph[w][kl];
#pragma unroll 4
        for (int t = 0; t < nbc; ++t) {
          const double2 f = phk[t];
          const int64_t o = s_off[w][t] + e;
          const double bh = blk_H[o], bs = blk_S[o];
          h.x = fma(bh, f.x, h.x);
          h.y = fma(bh, f.y, h.y);
          sv.x = fma(bs, f.x, sv.x);
          sv.y = fma(bs, f.y, sv.y);
        }
        if (last && diag && al == bl) {
          h.x += onsite[al];
          sv.x += 1.0;
        }
        H[dst] = h;
        S[dst] = sv;
      }
      if (last) break;
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
  const int64_t need = (n_units + BW - 1) / BW;      // one unit per warp
  if (need > 0x7fffffffLL) return SKN_ERR_CAPACITY;
  const unsigned grid = (unsigned)need;
  k_bloch_pairs<<<grid, BW * 32, 0, stream>>>(n_struct, n_units, unit_base, k_ptr, hs_off, atom_ptr, orb_ptr,
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
