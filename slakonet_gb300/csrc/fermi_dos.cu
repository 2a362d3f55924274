// Fermi level, band-gap statistics and Gaussian DOS, one CTA per structure.
//
// Fermi level.  The reference iterates mu <- mu - L / (dL/dmu + 1e-12) on
// L = (2 sum_k w_k sum_b f(e_kb; mu, kT) - Ne)^2 from mu0 = mean(e), with
// f = 1/(exp((e - mu)/kT) + 1) and dL/dmu taken by autograd, stopping once
// |dL/dmu| < tol or after max_iter updates (slakonet/fermi.py:139-215).
// Autograd's derivative of that expression is
//   dL/dmu = 2 (N - Ne) * 2 sum w f^2 exp(x) / kT,
// which is NaN as soon as one exp(x) overflows (0 * inf); the kernel keeps
// that product so divergent cases end in NaN exactly where the reference's do.
//
// Gap statistics follow calculate_band_gap (slakonet/main.py:637-707),
// calculate_band_structure_properties (slakonet/main.py:1539-1642) and the
// get_fermi extras (slakonet/optim.py:1011-1060); H2E = 27.211 eV/Ha
// (slakonet/main.py:34).
//
// DOS.  dos(E) = sum_k w_k sum_b exp(-((E - (e_kb - mu) H2E)/sigma)^2 / 2)
// / (sigma sqrt(2 pi)) on the torch.linspace grid (slakonet/main.py:709-797).
// Bands are ascending per k, so a binary search finds the bands within
// `window_sigmas` sigma of each grid point; one thread per grid point keeps
// the summation order fixed (no atomics).
#include "skn_common.cuh"

namespace {

constexpr double H2E = 27.211;
constexpr int NT = 256;

// stats layout (SKN_NSTAT doubles per structure)
enum {
  ST_MU_HA = 0, ST_FERMI_EV = 1, ST_GAP_EV = 2, ST_VBM_EV = 3, ST_CBM_EV = 4, ST_DIRECT = 5,
  ST_VBM_K = 6, ST_CBM_K = 7, ST_VWIDTH = 8, ST_CWIDTH = 9, ST_MIN_DGAP = 10, ST_DIRECT_SEMI = 11,
  ST_EFERMI_EV = 12, ST_BANDGAP_EV = 13, ST_CONVERGED = 14, ST_ITERS = 15, ST_DOS_FERMI = 16,
  ST_DOS_GAPC = 17, ST_DOS_TOTAL = 18, ST_METAL = 19, ST_FALLBACK = 20, ST_VBM_FLAT = 21, ST_CBM_FLAT = 22,
  ST_BAND_ENERGY = 23
};

__device__ __forceinline__ double qnan() { return __longlong_as_double(0x7ff8000000000000LL); }

struct Red {
  double v[NT / 32 * 4];
};

// block reductions for 2 sums
__device__ __forceinline__ void block_sum2(double& a, double& b, double* red) {
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) { red[w] = a; red[nw + w] = b; }
  __syncthreads();
  a = 0.0; b = 0.0;
  for (int i = 0; i < nw; ++i) { a += red[i]; b += red[nw + i]; }
}

// block max/min with first flat index of the extreme (ties: smallest index)
__device__ __forceinline__ void block_argext(double& v, int& idx, bool is_max, double* redv, int* redi) {
  for (int o = 16; o > 0; o >>= 1) {
    double ov = __shfl_xor_sync(0xffffffffu, v, o);
    int oi = __shfl_xor_sync(0xffffffffu, idx, o);
    bool take = is_max ? (ov > v || (ov == v && oi < idx)) : (ov < v || (ov == v && oi < idx));
    if (take) { v = ov; idx = oi; }
  }
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) { redv[w] = v; redi[w] = idx; }
  __syncthreads();
  v = redv[0]; idx = redi[0];
  for (int i = 1; i < nw; ++i) {
    bool take = is_max ? (redv[i] > v || (redv[i] == v && redi[i] < idx)) : (redv[i] < v || (redv[i] == v && redi[i] < idx));
    if (take) { v = redv[i]; idx = redi[i]; }
  }
}

__global__ void __launch_bounds__(NT) k_fermi_gap(const int64_t* __restrict__ eig_off, const int32_t* __restrict__ nkv,
                                                  const int32_t* __restrict__ nbv, const int64_t* __restrict__ kw_off,
                                                  const double* __restrict__ kweights, const double* __restrict__ nelec,
                                                  const double* __restrict__ eigall, double kT, double tol, int max_iter,
                                                  double* __restrict__ mu_out, double* __restrict__ stats,
                                                  int32_t* __restrict__ status) {
  __shared__ double red[4 * NT / 32];
  __shared__ int redi[NT / 32];
  const int s = blockIdx.x, tid = threadIdx.x;
  const int nk = nkv[s], nb = nbv[s];
  const int tot = nk * nb;
  const double* E = eigall + eig_off[s];
  const double* w = kweights + kw_off[s];
  const double ne = nelec[s];
  double* st = stats + (int64_t)SKN_NSTAT * s;

  // mu0 = mean(e)
  double a = 0.0, b = 0.0;
  for (int e = tid; e < tot; e += NT) a += E[e];
  block_sum2(a, b, red);
  double mu = a / (double)tot;
  int iters = max_iter, conv = 0;
  for (int it = 0; it < max_iter; ++it) {
    double sumo = 0.0, sumg = 0.0;
    for (int e = tid; e < tot; e += NT) {
      const double wk = w[e / nb];
      const double t3 = exp((E[e] - mu) / kT);
      const double occ = (1.0 / (t3 + 1.0)) * 1.0;
      sumo = fma(occ, wk, sumo);
      sumg += ((wk * occ) * occ) * t3;
    }
    block_sum2(sumo, sumg, red);
    const double total = 2.0 * sumo;
    const double diff = total - ne;
    const double loss = diff * diff;
    const double grad = (2.0 * (2.0 * diff)) * sumg / kT;
    if (fabs(grad) < tol) { iters = it; conv = 1; break; }
    mu = mu - loss / (grad + 1e-12);
  }

  // Fermi-smeared band energy, SimpleDftb._calculate_electronic_energy (slakonet/main.py:1430-1448):
  // sum_k w_k sum_b f(e_kb; mu, 0.025 eV) e_kb, with f = 0 where e_kb is exactly zero (fermi_smearing,
  // slakonet/fermi.py:54-96)
  {
    const double kT_e = 0.025 / H2E;
    double be = 0.0, unused = 0.0;
    for (int e = tid; e < tot; e += NT) {
      const double occ = (E[e] == 0.0) ? 0.0 : 1.0 / (1.0 + exp((E[e] - mu) / kT_e));
      be += (occ * E[e]) * w[e / nb];
    }
    block_sum2(be, unused, red);
    if (tid == 0) st[ST_BAND_ENERGY] = be;
  }

  // calculate_band_gap
  const double f_ev = mu * H2E;
  double vbm = -INFINITY, cbm = INFINITY;
  int vbi = 0x7fffffff, cbi = 0x7fffffff;
  int metal = 0, nocc = 0, nunocc = 0;
  for (int e = tid; e < tot; e += NT) {
    const double ev = E[e] * H2E;
    if (fabs(ev - f_ev) < 1e-3) metal = 1;
    if (ev < f_ev) { ++nocc; if (ev > vbm || (ev == vbm && e < vbi)) { vbm = ev; vbi = e; } }
    if (ev >= f_ev) { ++nunocc; if (ev < cbm || (ev == cbm && e < cbi)) { cbm = ev; cbi = e; } }
  }
  metal = __syncthreads_or(metal);
  nocc = __syncthreads_count(nocc > 0);
  nunocc = __syncthreads_count(nunocc > 0);
  block_argext(vbm, vbi, true, red, redi);
  block_argext(cbm, cbi, false, red, redi);

  // calculate_band_structure_properties on (e - mu) H2E
  double vmax = -INFINITY, vmin = INFINITY, cmax = -INFINITY, cmin = INFINITY;
  for (int e = tid; e < tot; e += NT) {
    const double ev = (E[e] - mu) * H2E;
    if (ev < 0.0) { vmax = fmax(vmax, ev); vmin = fmin(vmin, ev); }
    if (ev >= 0.0) { cmax = fmax(cmax, ev); cmin = fmin(cmin, ev); }
  }
  int dummy = 0;
  block_argext(vmax, dummy, true, red, redi);
  block_argext(vmin, dummy, false, red, redi);
  block_argext(cmax, dummy, true, red, redi);
  block_argext(cmin, dummy, false, red, redi);
  double dgap = INFINITY;
  for (int k = tid; k < nk; k += NT) {
    double kv = -INFINITY, kc = INFINITY;
    int hv = 0, hc = 0;
    for (int bb = 0; bb < nb; ++bb) {
      const double ev = (E[k * nb + bb] - mu) * H2E;
      if (ev < 0.0) { kv = fmax(kv, ev); hv = 1; }
      if (ev > 0.0) { kc = fmin(kc, ev); hc = 1; }
    }
    if (hv && hc) dgap = fmin(dgap, kc - kv);
  }
  block_argext(dgap, dummy, false, red, redi);

  // get_fermi extras: occ = e <= mu, unocc = e > mu
  double gv = -INFINITY, gc = INFINITY;
  for (int e = tid; e < tot; e += NT) {
    if (E[e] <= mu) gv = fmax(gv, E[e]);
    if (E[e] > mu) gc = fmin(gc, E[e]);
  }
  block_argext(gv, dummy, true, red, redi);
  block_argext(gc, dummy, false, red, redi);

  if (tid == 0) {
    mu_out[s] = mu;
    const bool vfound = vmax != -INFINITY, cfound = cmin != INFINITY;
    const double bs_gap = (vfound && cfound) ? (cmin - vmax) : 0.0;
    st[ST_VWIDTH] = vfound ? (vmax - vmin) : 0.0;
    st[ST_CWIDTH] = cfound ? (cmax - cmin) : 0.0;
    const bool dfound = dgap != INFINITY;
    st[ST_MIN_DGAP] = dfound ? dgap : qnan();
    st[ST_DIRECT_SEMI] = dfound ? (fabs(bs_gap - dgap) < 0.01 ? 1.0 : 0.0) : 0.0;
    st[ST_CONVERGED] = conv;
    st[ST_ITERS] = iters;
    st[ST_METAL] = metal;
    if (metal) {
      st[ST_MU_HA] = mu; st[ST_FERMI_EV] = mu * H2E; st[ST_GAP_EV] = 0.0;
      st[ST_VBM_EV] = f_ev; st[ST_CBM_EV] = f_ev; st[ST_DIRECT] = 0.0;
      st[ST_VBM_K] = 0; st[ST_CBM_K] = 0; st[ST_FALLBACK] = 0.0;
    } else if (nocc == 0 || nunocc == 0) {
      // the reference's empty max/min raises; get_properties_dict falls back to zeros
      st[ST_MU_HA] = 0.0; st[ST_FERMI_EV] = 0.0; st[ST_GAP_EV] = 0.0;
      st[ST_VBM_EV] = 0.0; st[ST_CBM_EV] = 0.0; st[ST_DIRECT] = 1.0;
      st[ST_VBM_K] = 0; st[ST_CBM_K] = 0; st[ST_FALLBACK] = 1.0;
    } else {
      st[ST_MU_HA] = mu; st[ST_FERMI_EV] = mu * H2E; st[ST_GAP_EV] = cbm - vbm;
      st[ST_VBM_EV] = vbm; st[ST_CBM_EV] = cbm;
      const int vk = vbi / nb, ck = cbi / nb;
      st[ST_DIRECT] = (vk == ck) ? 1.0 : 0.0;
      st[ST_VBM_K] = vk; st[ST_CBM_K] = ck; st[ST_FALLBACK] = 0.0;
    }
    st[ST_VBM_FLAT] = (metal || nocc == 0 || nunocc == 0) ? -1.0 : (double)vbi;
    st[ST_CBM_FLAT] = (metal || nocc == 0 || nunocc == 0) ? -1.0 : (double)cbi;
    st[ST_EFERMI_EV] = mu * H2E;
    const double bg = gc - gv;
    st[ST_BANDGAP_EV] = (bg > 0.0 ? bg : (bg == bg ? 0.0 : bg)) * H2E;
    status[s] = conv ? SKN_OK : SKN_ERR_NO_CONVERGE;
  }
}

// torch.linspace grid: fma(step, i, lo) for the first half, fma(-step, n-1-i, hi) after.
__device__ __forceinline__ double lin_grid(double lo, double hi, int n, int i) {
  if (n == 1) return lo;
  const double step = (hi - lo) / (double)(n - 1);
  return (i < n / 2) ? fma(step, (double)i, lo) : fma(-step, (double)(n - 1 - i), hi);
}

__global__ void __launch_bounds__(NT) k_dos(const int64_t* __restrict__ eig_off, const int32_t* __restrict__ nkv,
                                            const int32_t* __restrict__ nbv, const int64_t* __restrict__ kw_off,
                                            const double* __restrict__ kweights, const double* __restrict__ eigall,
                                            const double* __restrict__ muv, double e_lo, double e_hi, int npts,
                                            double sigma, double window, double* __restrict__ grid,
                                            double* __restrict__ dos) {
  const int s = blockIdx.y;
  const int i = blockIdx.x * NT + threadIdx.x;
  if (i >= npts) return;
  const double x = lin_grid(e_lo, e_hi, npts, i);
  if (s == 0) grid[i] = x;
  const int nk = nkv[s], nb = nbv[s];
  const double* E = eigall + eig_off[s];
  const double* w = kweights + kw_off[s];
  const double mu = muv[s];
  const double inv_sigma = 1.0 / sigma;
  const double inv_norm = 1.0 / (sigma * sqrt(2.0 * 3.141592653589793));
  double acc = 0.0;
  if (!(mu == mu)) {
    acc = qnan();
  } else if (window > 0.0) {
    const double lo = x - window * sigma, hi = x + window * sigma;
    for (int k = 0; k < nk; ++k) {
      const double* Ek = E + (int64_t)k * nb;
      // first band with (e - mu) H2E >= lo
      int a = 0, b = nb;
      while (a < b) {
        const int m = (a + b) >> 1;
        if ((Ek[m] - mu) * H2E < lo) a = m + 1; else b = m;
      }
      double sk = 0.0;
      for (int bb = a; bb < nb; ++bb) {
        const double ev = (Ek[bb] - mu) * H2E;
        if (ev > hi) break;
        const double t = (x - ev) * inv_sigma;
        sk += exp(-0.5 * (t * t)) * inv_norm;
      }
      acc = fma(w[k], sk, acc);
    }
  } else {
    for (int k = 0; k < nk; ++k) {
      const double* Ek = E + (int64_t)k * nb;
      double sk = 0.0;
      for (int bb = 0; bb < nb; ++bb) {
        const double t = (x - (Ek[bb] - mu) * H2E) * inv_sigma;
        sk += exp(-0.5 * (t * t)) * inv_norm;
      }
      acc = fma(w[k], sk, acc);
    }
  }
  dos[(int64_t)s * npts + i] = acc;
}

// The windowed DOS with fewer exponentials.  A thread owns DG consecutive grid points and an eighth of
// the k-points (k = kg, kg + 8, ...).  Along the grid a Gaussian obeys g(x + D) = g(x) f(x) and
// f(x + D) = f(x) r, with t = (x - e) / sigma, d = D / sigma, f = exp(-(t d + d^2 / 2)) and
// r = exp(-d^2); so a band costs two exponentials at the first grid point inside its window and two
// multiplications per further point, instead of one exponential per point.  A point takes a band
// exactly when k_dos would (the same window test on the same values); the recurrence starts inside the
// window (|t| <= window), so it neither underflows nor loses the points it serves.  The eight k-point
// groups are added in a fixed order, so the result depends on the structure alone.
constexpr int DG = 8;                  // grid points per thread
constexpr int DKG = 8;                 // k-point groups per chunk of grid points
constexpr int DCH = NT / DKG;          // chunks per CTA

__global__ void __launch_bounds__(NT) k_dos_win(const int64_t* __restrict__ eig_off, const int32_t* __restrict__ nkv,
                                                const int32_t* __restrict__ nbv, const int64_t* __restrict__ kw_off,
                                                const double* __restrict__ kweights, const double* __restrict__ eigall,
                                                const double* __restrict__ muv, double e_lo, double e_hi, int npts,
                                                double sigma, double window, double* __restrict__ grid,
                                                double* __restrict__ dos) {
  __shared__ double part[DKG][DCH][DG];
  const int s = blockIdx.y;
  const int kg = threadIdx.x / DCH, cl = threadIdx.x % DCH;
  const int i0 = (blockIdx.x * DCH + cl) * DG;
  const int cnt = max(0, min(DG, npts - i0));
  double x[DG], acc[DG];
#pragma unroll
  for (int j = 0; j < DG; ++j) {
    x[j] = lin_grid(e_lo, e_hi, npts, min(i0 + j, npts - 1));
    acc[j] = 0.0;
  }
  if (s == 0 && kg == 0) {
#pragma unroll
    for (int j = 0; j < DG; ++j)
      if (j < cnt) grid[i0 + j] = x[j];
  }
  const int nk = nkv[s], nb = nbv[s];
  const double* E = eigall + eig_off[s];
  const double* w = kweights + kw_off[s];
  const double mu = muv[s];
  const double inv_sigma = 1.0 / sigma;
  const double inv_norm = 1.0 / (sigma * sqrt(2.0 * 3.141592653589793));
  const double d = (npts > 1 ? (e_hi - e_lo) / (double)(npts - 1) : 0.0) * inv_sigma;
  const double r = exp(-d * d);
  const bool nan_mu = !(mu == mu);
  if (cnt > 0 && !nan_mu) {
    const double lo0 = x[0] - window * sigma;
    const double hi_last = lin_grid(e_lo, e_hi, npts, i0 + cnt - 1) + window * sigma;   // the chunk's last point
    for (int k = kg; k < nk; k += DKG) {
      const double* Ek = E + (int64_t)k * nb;
      int a = 0, b = nb;                       // first band with (e - mu) H2E >= the first point's window
      while (a < b) {
        const int m = (a + b) >> 1;
        if ((Ek[m] - mu) * H2E < lo0) a = m + 1; else b = m;
      }
      double sk[DG];
#pragma unroll
      for (int j = 0; j < DG; ++j) sk[j] = 0.0;
      for (int bb = a; bb < nb; ++bb) {
        const double ev = (Ek[bb] - mu) * H2E;
        if (ev > hi_last) break;
        // the points whose window holds ev form one run [j0, j1] (the grid ascends); the same tests as k_dos
        int j0 = DG, j1 = -1;
        double xs = x[0];
#pragma unroll
        for (int j = 0; j < DG; ++j) {
          const bool in = j < cnt && ev >= x[j] - window * sigma && ev <= x[j] + window * sigma;
          if (in && j0 == DG) {
            j0 = j;
            xs = x[j];
          }
          if (in) j1 = j;
        }
        if (j1 < 0) continue;
        // both exponentials at the run's first point, every lane together
        const double t = (xs - ev) * inv_sigma;
        double g = exp(-0.5 * (t * t));
        double f = exp(-fma(t, d, 0.5 * d * d));
#pragma unroll
        for (int j = 0; j < DG; ++j) {
          if (j >= j0 && j <= j1) {
            sk[j] += g * inv_norm;
            g *= f;
            f *= r;
          }
        }
      }
#pragma unroll
      for (int j = 0; j < DG; ++j) acc[j] = fma(w[k], sk[j], acc[j]);
    }
  }
#pragma unroll
  for (int j = 0; j < DG; ++j) part[kg][cl][j] = acc[j];
  __syncthreads();
  if (kg == 0) {
    for (int j = 0; j < cnt; ++j) {
      double v = part[0][cl][j];
#pragma unroll
      for (int q = 1; q < DKG; ++q) v += part[q][cl][j];
      dos[(int64_t)s * npts + i0 + j] = nan_mu ? qnan() : v;
    }
  }
}

// dos_at_fermi (grid point closest to 0), gap centre (DOS minimum within |E| < 2 eV)
// and trapezoid integral, as get_properties_dict (slakonet/main.py:1766-1782).
__global__ void __launch_bounds__(NT) k_dos_stats(const double* __restrict__ grid, const double* __restrict__ dos,
                                                  int npts, double* __restrict__ stats) {
  __shared__ double red[4 * NT / 32];
  __shared__ int redi[NT / 32];
  const int s = blockIdx.x, tid = threadIdx.x;
  const double* D = dos + (int64_t)s * npts;
  double av = INFINITY, mv = INFINITY, tr = 0.0, dummy = 0.0;
  int ai = 0x7fffffff, mi = 0x7fffffff;
  for (int i = tid; i < npts; i += NT) {
    const double g = grid[i];
    const double ag = fabs(g);
    if (ag < av || (ag == av && i < ai)) { av = ag; ai = i; }
    if (ag < 2.0 && (D[i] < mv || (D[i] == mv && i < mi))) { mv = D[i]; mi = i; }
    if (i + 1 < npts) tr += (grid[i + 1] - g) * (D[i] + D[i + 1]) * 0.5;
  }
  block_argext(av, ai, false, red, redi);
  block_argext(mv, mi, false, red, redi);
  block_sum2(tr, dummy, red);
  if (tid == 0) {
    double* st = stats + (int64_t)SKN_NSTAT * s;
    st[ST_DOS_FERMI] = D[ai];
    st[ST_DOS_GAPC] = (mi < npts) ? grid[mi] : qnan();
    st[ST_DOS_TOTAL] = tr;
  }
}

}  // namespace

extern "C" int skn_fermi_gap(int n_struct, const int64_t* eig_off, const int32_t* nk, const int32_t* nb,
                             const int64_t* kw_off, const double* kweights, const double* nelec, const double* eig,
                             double kT, double tol, int max_iter, double* mu, double* stats, int32_t* status,
                             cudaStream_t stream) {
  if (n_struct < 0 || max_iter < 0 || !(kT > 0.0)) return SKN_ERR_ARG;
  if (n_struct == 0) return SKN_OK;
  if (!eig_off || !nk || !nb || !kw_off || !kweights || !nelec || !eig || !mu || !stats || !status)
    return SKN_ERR_ARG;
  k_fermi_gap<<<n_struct, NT, 0, stream>>>(eig_off, nk, nb, kw_off, kweights, nelec, eig, kT, tol, max_iter, mu,
                                           stats, status);
  return cudaPeekAtLastError() == cudaSuccess ? SKN_OK : SKN_ERR_CUDA;
}

extern "C" int skn_dos(int n_struct, const int64_t* eig_off, const int32_t* nk, const int32_t* nb,
                       const int64_t* kw_off, const double* kweights, const double* eig, const double* mu,
                       double e_lo, double e_hi, int npts, double sigma, double window_sigmas, double* grid,
                       double* dos, double* stats, cudaStream_t stream) {
  if (n_struct < 0 || npts <= 0 || !(sigma > 0.0) || window_sigmas < 0.0) return SKN_ERR_ARG;
  if (n_struct == 0) return SKN_OK;
  if (!eig_off || !nk || !nb || !kw_off || !kweights || !eig || !mu || !grid || !dos || !stats) return SKN_ERR_ARG;
  if (n_struct > 65535) return SKN_ERR_CAPACITY;
  if (window_sigmas > 0.0) {
    dim3 g((npts + DCH * DG - 1) / (DCH * DG), n_struct);
    k_dos_win<<<g, NT, 0, stream>>>(eig_off, nk, nb, kw_off, kweights, eig, mu, e_lo, e_hi, npts, sigma,
                                    window_sigmas, grid, dos);
  } else {
    dim3 g((npts + NT - 1) / NT, n_struct);
    k_dos<<<g, NT, 0, stream>>>(eig_off, nk, nb, kw_off, kweights, eig, mu, e_lo, e_hi, npts, sigma, window_sigmas,
                                grid, dos);
  }
  if (cudaPeekAtLastError() != cudaSuccess) return SKN_ERR_CUDA;
  k_dos_stats<<<n_struct, NT, 0, stream>>>(grid, dos, npts, stats);
  return cudaPeekAtLastError() == cudaSuccess ? SKN_OK : SKN_ERR_CUDA;
}

extern "C" int skn_abi_version(void) { return 100; }
