// Neighbour list / bond table and Bloch phases.
//
// A bond is a directed triple (i, j, T): atom i of the home cell, atom j of
// the cell translated by the integer vector T, with 0 < |r_j + T.cell - r_i|
// < cutoff.  This is the set the reference selects from its dense
// [cells, N, N] distance tables (slakonet/atoms.py:217-243) with the mask
// of hs_matrix (slakonet/slaterkoster.py:269-276).  Here one thread walks
// the translation box of one ordered atom pair; distances are screened in
// FP32 (73x the FP64 rate on GB300) and every candidate near or inside the
// cutoff is decided and measured in FP64.
#include "skn_common.cuh"

namespace {

struct PairCtx {
  int s, i, j, N, a0;
};

__device__ __forceinline__ int find_struct(const int64_t* base, int n, int64_t e) {
  // largest s with base[s] <= e
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (base[mid] <= e) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Walk all translations of pair (i, j) in x-slowest order; call f(tlin, d, v) for each bond.
template <typename F>
__device__ __forceinline__ void walk_pair(const double* cell, const double* ri, const double* rj,
                                          const int32_t* rng, double cutoff, F&& f) {
  const int r0 = rng[0], r1 = rng[1], r2 = rng[2];
  const int w1 = 2 * r1 + 1, w2 = 2 * r2 + 1;
  float cf[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) cf[q] = (float)cell[q];
  const float dx = (float)(rj[0] - ri[0]), dy = (float)(rj[1] - ri[1]), dz = (float)(rj[2] - ri[2]);
  const float lim = (float)(cutoff + 0.01);
  const float lim2 = lim * lim;
  for (int t0 = -r0; t0 <= r0; ++t0) {
    for (int t1 = -r1; t1 <= r1; ++t1) {
      for (int t2 = -r2; t2 <= r2; ++t2) {
        float vx = fmaf((float)t0, cf[0], fmaf((float)t1, cf[3], fmaf((float)t2, cf[6], dx)));
        float vy = fmaf((float)t0, cf[1], fmaf((float)t1, cf[4], fmaf((float)t2, cf[7], dy)));
        float vz = fmaf((float)t0, cf[2], fmaf((float)t1, cf[5], fmaf((float)t2, cf[8], dz)));
        float d2 = fmaf(vx, vx, fmaf(vy, vy, vz * vz));
        if (d2 >= lim2) continue;
        // FP64: image position (T . cell + r_j) minus r_i, as the reference forms it.
        double v[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          double tc = fma((double)t2, cell[6 + a], fma((double)t1, cell[3 + a], (double)t0 * cell[a]));
          v[a] = (tc + rj[a]) - ri[a];
        }
        double d = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        if (d < cutoff && d > 0.0) {
          int tlin = ((t0 + r0) * w1 + (t1 + r1)) * w2 + (t2 + r2);
          f(tlin, d, v);
        }
      }
    }
  }
}

__global__ void k_bond_counts(int n_struct, const int32_t* __restrict__ atom_ptr,
                              const double* __restrict__ pos, const double* __restrict__ cells,
                              const int32_t* __restrict__ image_range, double cutoff,
                              const int64_t* __restrict__ pair_base, int64_t n_pairs,
                              int32_t* __restrict__ counts) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n_pairs;
       e += (int64_t)gridDim.x * blockDim.x) {
    int s = find_struct(pair_base, n_struct, e);
    int a0 = atom_ptr[s], N = atom_ptr[s + 1] - a0;
    int64_t loc = e - pair_base[s];
    int i = (int)(loc / N), j = (int)(loc % N);
    int c = 0;
    walk_pair(cells + 9 * s, pos + 3 * (a0 + i), pos + 3 * (a0 + j), image_range + 3 * s, cutoff,
              [&](int, double, const double*) { ++c; });
    counts[e] = c;
  }
}

__global__ void k_bond_fill(int n_struct, const int32_t* __restrict__ atom_ptr,
                            const double* __restrict__ pos, const double* __restrict__ cells,
                            const int32_t* __restrict__ image_range, double cutoff,
                            const int64_t* __restrict__ pair_base, int64_t n_pairs,
                            const int64_t* __restrict__ pair_ptr, const int64_t* __restrict__ pair_blk_base,
                            const int32_t* __restrict__ atom_norb, int32_t* __restrict__ bond_i,
                            int32_t* __restrict__ bond_j, int32_t* __restrict__ bond_img,
                            double* __restrict__ bond_d, double* __restrict__ bond_u,
                            int64_t* __restrict__ bond_blk) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n_pairs;
       e += (int64_t)gridDim.x * blockDim.x) {
    int s = find_struct(pair_base, n_struct, e);
    int a0 = atom_ptr[s], N = atom_ptr[s + 1] - a0;
    int64_t loc = e - pair_base[s];
    int i = (int)(loc / N), j = (int)(loc % N);
    const int gi = a0 + i, gj = a0 + j;
    const int64_t bsz = (int64_t)atom_norb[gi] * atom_norb[gj];
    int64_t b = pair_ptr[e];
    int64_t blk = pair_blk_base[e];
    walk_pair(cells + 9 * s, pos + 3 * gi, pos + 3 * gj, image_range + 3 * s, cutoff,
              [&](int tlin, double d, const double* v) {
                bond_i[b] = gi;
                bond_j[b] = gj;
                bond_img[b] = tlin;
                bond_d[b] = d;
                bond_u[3 * b + 0] = v[0] / d;
                bond_u[3 * b + 1] = v[1] / d;
                bond_u[3 * b + 2] = v[2] / d;
                bond_blk[b] = blk;
                ++b;
                blk += bsz;
              });
  }
}

__global__ void k_image_phases(const int32_t* __restrict__ image_range, const int32_t* __restrict__ k_ptr,
                               const double* __restrict__ kpoints, const int64_t* __restrict__ phase_base,
                               double2* __restrict__ phases) {
  const int s = blockIdx.y;
  const int r0 = image_range[3 * s], r1 = image_range[3 * s + 1], r2 = image_range[3 * s + 2];
  const int w1 = 2 * r1 + 1, w2 = 2 * r2 + 1;
  const int nimg = (2 * r0 + 1) * w1 * w2;
  const int k0 = k_ptr[s], nk = k_ptr[s + 1] - k0;
  const int64_t total = (int64_t)nk * nimg;
  double2* out = phases + phase_base[s];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int k = (int)(e / nimg), t = (int)(e % nimg);
    int t2 = t % w2 - r2, t1 = (t / w2) % w1 - r1, t0 = t / (w1 * w2) - r0;
    const double* kk = kpoints + 3 * (k0 + k);
    // exp(i 2 pi k.T) = cospi(2 k.T) + i sinpi(2 k.T)
    double x = 2.0 * (kk[0] * t0 + kk[1] * t1 + kk[2] * t2);
    double sn, cs;
    sincospi(x, &sn, &cs);
    out[e] = make_double2(cs, sn);
  }
}

}  // namespace

extern "C" int skn_bond_counts(int n_struct, int64_t n_pairs, const int32_t* atom_ptr, const double* positions,
                                 const double* cells, const int32_t* image_range, double cutoff,
                                 const int64_t* pair_base, int32_t* pair_counts, cudaStream_t stream) {
  if (n_struct <= 0 || n_pairs < 0 || !atom_ptr || !positions || !cells || !image_range || !pair_base || !pair_counts)
    return n_struct == 0 ? SKN_OK : SKN_ERR_ARG;
  if (n_pairs == 0) return SKN_OK;
  int threads = 128;
  int64_t blocks = (n_pairs + threads - 1) / threads;
  if (blocks > 152 * 64) blocks = 152 * 64;
  k_bond_counts<<<(unsigned)blocks, threads, 0, stream>>>(n_struct, atom_ptr, positions, cells, image_range,
                                                          cutoff, pair_base, n_pairs, pair_counts);
  return cudaPeekAtLastError() == cudaSuccess ? SKN_OK : SKN_ERR_CUDA;
}

extern "C" int skn_bond_fill(int n_struct, int64_t n_pairs, const int32_t* atom_ptr, const double* positions,
                               const double* cells, const int32_t* image_range, double cutoff,
                               const int64_t* pair_base, const int64_t* pair_ptr, const int64_t* pair_blk_base,
                               const int32_t* atom_norb, int32_t* bond_i, int32_t* bond_j, int32_t* bond_img,
                               double* bond_d, double* bond_u, int64_t* bond_blk, cudaStream_t stream) {
  if (n_struct <= 0 || n_pairs < 0) return n_struct == 0 ? SKN_OK : SKN_ERR_ARG;
  if (!atom_ptr || !positions || !cells || !image_range || !pair_base || !pair_ptr || !pair_blk_base ||
      !atom_norb || !bond_i || !bond_j || !bond_img || !bond_d || !bond_u || !bond_blk)
    return SKN_ERR_ARG;
  if (n_pairs == 0) return SKN_OK;
  int threads = 128;
  int64_t blocks = (n_pairs + threads - 1) / threads;
  if (blocks > 152 * 64) blocks = 152 * 64;
  k_bond_fill<<<(unsigned)blocks, threads, 0, stream>>>(n_struct, atom_ptr, positions, cells, image_range, cutoff,
                                                        pair_base, n_pairs, pair_ptr, pair_blk_base, atom_norb,
                                                        bond_i, bond_j, bond_img, bond_d, bond_u, bond_blk);
  return cudaPeekAtLastError() == cudaSuccess ? SKN_OK : SKN_ERR_CUDA;
}

extern "C" int skn_image_phases(int n_struct, const int32_t* image_range, const int32_t* k_ptr,
                                const double* kpoints, const int64_t* phase_base, double* phases,
                                cudaStream_t stream) {
  if (n_struct < 0) return SKN_ERR_ARG;
  if (n_struct == 0) return SKN_OK;
  if (!image_range || !k_ptr || !kpoints || !phase_base || !phases) return SKN_ERR_ARG;
  if (n_struct > 65535) return SKN_ERR_CAPACITY;
  dim3 grid(64, n_struct);
  k_image_phases<<<grid, 128, 0, stream>>>(image_range, k_ptr, kpoints, phase_base, (double2*)phases);
  return cudaPeekAtLastError() == cudaSuccess ? SKN_OK : SKN_ERR_CUDA;
}
