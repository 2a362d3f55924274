// Atom-type projected DOS from eigenvectors with Gaussian broadening.
//
// Replaces compute_atom_projected_dos (slakonet/predict_slakonet.py:119-210),
// which loops over (k, band) in Python.  Two launches:
//   k_pdos_weights  thread per (k, band): w[k][b][g] = sum_{i in group g} |c_ib|^2
//                   (rows i of the eigenvector matrix are read across
//                   consecutive bands, so warps load contiguous memory);
//   k_pdos          thread per (group, grid point): sum over k, then band, of
//                   w * exp(-0.5 ((E - e_kb) / sigma)^2) / (sigma sqrt(2 pi)),
//                   divided by nk, on the torch.linspace grid shifted by E_F.
// The products and sums are rounded separately (no contraction), in the
// reference's (k, band) order.
#include "skn_common.cuh"

namespace {

constexpr int PT = 128;

__global__ void __launch_bounds__(PT) k_pdos_weights(int nk, int nb, int n_orb, const double2* __restrict__ vec,
                                                     const int32_t* __restrict__ group, int n_group,
                                                     double* __restrict__ w) {
  const int64_t t = (int64_t)blockIdx.x * PT + threadIdx.x;
  if (t >= (int64_t)nk * nb) return;
  const int k = (int)(t / nb), b = (int)(t % nb);
  const double2* v = vec + (int64_t)k * n_orb * nb + b;
  for (int g = 0; g < n_group; ++g) {
    double s = 0.0;
    for (int i = 0; i < n_orb; ++i) {
      if (group[i] != g) continue;
      const double2 c = v[(int64_t)i * nb];
      s = __dadd_rn(s, __dadd_rn(__dmul_rn(c.x, c.x), __dmul_rn(c.y, c.y)));
    }
    w[t * n_group + g] = s;
  }
}

// torch.linspace grid: fma(step, i, lo) for the first half, fma(-step, n-1-i, hi) after.
__device__ __forceinline__ double lin_grid(double lo, double hi, int n, int i) {
  if (n == 1) return lo;
  const double step = (hi - lo) / (double)(n - 1);
  return (i < n / 2) ? fma(step, (double)i, lo) : fma(-step, (double)(n - 1 - i), hi);
}

__global__ void __launch_bounds__(PT) k_pdos(int nk, int nb, const double* __restrict__ eig,
                                             const double* __restrict__ w, int n_group, double fermi_ev,
                                             double e_lo, double e_hi, int npts, double sigma, double h2e,
                                             double* __restrict__ grid, double* __restrict__ pdos) {
  const int e = blockIdx.x * PT + threadIdx.x;
  const int g = blockIdx.y;
  if (e >= npts) return;
  const double x = lin_grid(e_lo, e_hi, npts, e);
  if (g == 0) grid[e] = x;
  const double xe = __dadd_rn(x, fermi_ev);
  const double norm = 1.0 / (sigma * sqrt(2.0 * 3.141592653589793));
  double acc = 0.0;
  for (int k = 0; k < nk; ++k) {
    for (int b = 0; b < nb; ++b) {
      const int64_t kb = (int64_t)k * nb + b;
      const double d = __dadd_rn(xe, -__dmul_rn(eig[kb], h2e)) / sigma;
      const double gauss = __dmul_rn(norm, exp(__dmul_rn(-0.5, __dmul_rn(d, d))));
      acc = __dadd_rn(acc, __dmul_rn(w[kb * n_group + g], gauss));
    }
  }
  pdos[(int64_t)g * npts + e] = acc / (double)nk;
}

}  // namespace

extern "C" int skn_atom_pdos(int nk, int nb, int n_orb, const double* eig, const double* vec,
                             const int32_t* orb_group, int n_group, double fermi_ev, double e_lo, double e_hi,
                             int npts, double sigma, double h2e, double* weights, double* grid, double* pdos,
                             cudaStream_t stream) {
  if (nk < 0 || nb < 0 || n_orb < 0 || n_group < 1 || npts < 1 || !(sigma > 0.0)) return SKN_ERR_ARG;
  if (!eig || !vec || !orb_group || !weights || !grid || !pdos) return SKN_ERR_ARG;
  if (n_group > 65535) return SKN_ERR_CAPACITY;
  const int64_t nkb = (int64_t)nk * nb;
  if (nkb > 0) {
    k_pdos_weights<<<(unsigned)((nkb + PT - 1) / PT), PT, 0, stream>>>(nk, nb, n_orb, (const double2*)vec,
                                                                      orb_group, n_group, weights);
    if (cudaPeekAtLastError() != cudaSuccess) return SKN_ERR_CUDA;
  }
  k_pdos<<<dim3((npts + PT - 1) / PT, n_group), PT, 0, stream>>>(nk > 0 ? nk : 1, nkb > 0 ? nb : 0, eig, weights,
                                                                  n_group, fermi_ev, e_lo, e_hi, npts, sigma, h2e,
                                                                  grid, pdos);
  return cudaPeekAtLastError() == cudaSuccess ? SKN_OK : SKN_ERR_CUDA;
}
