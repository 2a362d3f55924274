// Batched generalized Hermitian eigenvalues, FP64, one CTA per problem.
//
// For each (structure, k) problem H x = e S x the CTA runs
//   1. Cholesky S = L L^H (lower, right-looking, in place),
//   2. reduction to C = L^-1 H L^-H (LAPACK zhegs2 order: scale, axpy,
//      her2, axpy, triangular solve per column),
//   3. Householder tridiagonalisation of C (zhetd2: larfg, hemv, her2),
//   4. eigenvalues of the real tridiagonal by Sturm-count bisection, one
//      thread per eigenvalue, which returns them in ascending order.
// The reference runs torch.linalg.cholesky / solve / matmul / eigh per k
// (slakonet/utils.py:741-783) in a serial Python loop (slakonet/main.py:174).
//
// GB300 notes.  FP64 runs at ~1 TFLOP/s per GPU and a warp FP64 instruction
// costs the same with one or 32 lanes, so all O(n^2)-per-step loops map
// full warps onto contiguous work (packed-triangle indexing for the rank-2
// updates, rows-on-lanes with a uniform trip count for the hemv).  The CTA is
// persistent and pulls problems from a largest-first queue so big and small
// problems share every SM; several CTAs per SM hide the latency of the
// per-column scalar steps.  Problems with n <= SMEM_N are staged in shared
// memory; larger ones are factorised in place in global memory (L2-resident).
#include "skn_common.cuh"

namespace {

constexpr int NT = 256;           // threads per CTA
constexpr int NW = NT / 32;
constexpr int SMEM_N = 40;        // problems up to this size run from shared memory
constexpr int SMEM_LDA = SMEM_N + 1;
constexpr int MAX_N = 2048;       // shared-memory vectors bound the single-CTA path

struct Vecs {
  double2* w;      // n: hemv result / Householder w
  double* d;       // n: tridiagonal diagonal
  double* e2;      // n: squared off-diagonal (e2[i] couples i and i+1)
  double* rdiag;   // n: 1 / L[i][i]
  double* red;     // 4 * NW reduction scratch
  double* sc;      // 16 scalars
  float* d32;      // n: FP32 copy of d (aliases rdiag, free after the reduction)
  float* e232;     // n: FP32 copy of e^2
};

__device__ __forceinline__ double2 ld(const double2* A, int lda, int i, int j) { return A[i + (int64_t)j * lda]; }
__device__ __forceinline__ void st(double2* A, int lda, int i, int j, double2 v) { A[i + (int64_t)j * lda] = v; }

// Hermitian A (lower stored), rows >= r0: returns conj-aware element (i, j) of the full matrix.
__device__ __forceinline__ double2 herm(const double2* A, int lda, int i, int j) {
  const bool up = j > i;
  double2 v = up ? A[j + (int64_t)i * lda] : A[i + (int64_t)j * lda];
  v.y = cond_flip(v.y, up);
  return v;
}

// ---------------------------------------------------------------- Cholesky
__device__ bool cholesky_lower(double2* A, int lda, int n, Vecs& V) {
  const int tid = threadIdx.x;
  for (int k = 0; k < n; ++k) {
    if (tid == 0) {
      const double a = A[k + (int64_t)k * lda].x;
      const bool ok = (a > 0.0) && is_finite_bits(a);
      const double dk = ok ? sqrt(a) : 1.0;
      const double rd = 1.0 / dk;
      A[k + (int64_t)k * lda] = make_double2(dk, 0.0);
      V.rdiag[k] = rd;
      V.sc[0] = ok ? rd : 0.0;
      reinterpret_cast<int*>(V.sc)[2] = ok ? 0 : 1;
    }
    __syncthreads();
    if (reinterpret_cast<int*>(V.sc)[2]) return false;
    const double rd = V.sc[0];
    const int m = n - k - 1;
    for (int i = tid; i < m; i += NT) {
      double2 v = A[(k + 1 + i) + (int64_t)k * lda];
      A[(k + 1 + i) + (int64_t)k * lda] = cscale(v, rd);
    }
    __syncthreads();
    // trailing update of the packed lower triangle (k < j <= i)
    const int tri = m * (m + 1) / 2;
    for (int e = tid; e < tri; e += NT) {
      int ii, jj;
      tri_index(e, m, ii, jj);
      const int i = k + 1 + ii, j = k + 1 + jj;
      const double2 aik = A[i + (int64_t)k * lda];
      const double2 ajk = A[j + (int64_t)k * lda];
      A[i + (int64_t)j * lda] = cfms_conj(aik, ajk, A[i + (int64_t)j * lda]);
    }
    __syncthreads();
  }
  return true;
}

// y[i] = sum_j Herm(A)[r0+i][r0+j] x[j] for i < m, x and y in shared/global memory.
// Rows on lanes with a uniform trip count over j; when fewer than NT rows,
// warps split the j range and partial sums are added through `y` + red.
__device__ void hemv_lower(const double2* A, int lda, int r0, int m, const double2* x, double2* y, double2 scale,
                           double* red_c /* 2*NT doubles of scratch */) {
  const int tid = threadIdx.x;
  const int row_warps = (m + 31) >> 5;
  if (row_warps >= NW) {
    for (int i = tid; i < m; i += NT) {
      double2 acc = make_double2(0.0, 0.0);
      const int gi = r0 + i;
      for (int j = 0; j < m; ++j) acc = cfma(herm(A, lda, gi, r0 + j), x[j], acc);
      y[i] = cmul(scale, acc);
    }
    __syncthreads();
    return;
  }
  const int nsplit = NW / row_warps;
  const int w = tid >> 5, lane = tid & 31;
  const int rb = w % row_warps, sp = w / row_warps;
  const int i = rb * 32 + lane;
  double2 acc = make_double2(0.0, 0.0);
  if (sp < nsplit) {
    const int chunk = (m + nsplit - 1) / nsplit;
    const int j0 = sp * chunk, j1 = min(m, j0 + chunk);
    const int gi = r0 + min(i, m - 1);
    for (int j = j0; j < j1; ++j) acc = cfma(herm(A, lda, gi, r0 + j), x[j], acc);
  }
  double2* part = reinterpret_cast<double2*>(red_c);
  part[tid] = acc;
  __syncthreads();
  for (int r = tid; r < m; r += NT) {
    double2 s = make_double2(0.0, 0.0);
    const int rbw = r >> 5, ln = r & 31;
    for (int q = 0; q < nsplit; ++q) {
      const double2 v = part[(q * row_warps + rbw) * 32 + ln];
      s.x += v.x;
      s.y += v.y;
    }
    y[r] = cmul(scale, s);
  }
  __syncthreads();
}

// A22 -= x y^H + y x^H on the packed lower triangle of rows/cols r0..r0+m-1.
__device__ void her2_lower(double2* A, int lda, int r0, int m, const double2* x, int xinc_lda_col,
                           const double2* y) {
  (void)xinc_lda_col;
  const int tri = m * (m + 1) / 2;
  for (int e = threadIdx.x; e < tri; e += NT) {
    int ii, jj;
    tri_index(e, m, ii, jj);
    const int i = r0 + ii, j = r0 + jj;
    double2 a = A[i + (int64_t)j * lda];
    a = cfms_conj(x[ii], y[jj], a);
    a = cfms_conj(y[ii], x[jj], a);
    A[i + (int64_t)j * lda] = a;
  }
}

// ------------------------------------------------- reduction to standard form
// A (lower) <- L^-1 A L^-H with B = L from cholesky_lower (rdiag holds 1/L_kk).
__device__ void hegs2_lower(double2* A, int lda, const double2* B, int ldb, int n, Vecs& V) {
  const int tid = threadIdx.x;
  for (int k = 0; k < n; ++k) {
    if (tid == 0) {
      const double rd = V.rdiag[k];
      const double akk = A[k + (int64_t)k * lda].x * (rd * rd);
      A[k + (int64_t)k * lda] = make_double2(akk, 0.0);
      V.sc[0] = -0.5 * akk;
    }
    __syncthreads();
    const int m = n - k - 1;
    if (m == 0) break;
    const double ct = V.sc[0];
    const double rd = V.rdiag[k];
    double2* a = A + (k + 1) + (int64_t)k * lda;       // column k below the diagonal
    const double2* b = B + (k + 1) + (int64_t)k * ldb;
    for (int i = tid; i < m; i += NT) {
      double2 v = cscale(a[i], rd);
      v.x = fma(ct, b[i].x, v.x);
      v.y = fma(ct, b[i].y, v.y);
      a[i] = v;
    }
    __syncthreads();
    her2_lower(A, lda, k + 1, m, a, 0, b);
    __syncthreads();
    for (int i = tid; i < m; i += NT) {
      double2 v = a[i];
      v.x = fma(ct, b[i].x, v.x);
      v.y = fma(ct, b[i].y, v.y);
      a[i] = v;
    }
    __syncthreads();
    // forward substitution a <- L22^-1 a, in chunks of 32 rows: warp 0 solves the
    // diagonal chunk, then all threads apply it to the rows below.
    for (int c0 = 0; c0 < m; c0 += 32) {
      const int cm = min(32, m - c0);
      if (tid < 32) {
        const int lane = tid;
        double2 x = (lane < cm) ? a[c0 + lane] : make_double2(0.0, 0.0);
        for (int i = 0; i < cm; ++i) {
          double2 xi;
          if (lane == i) {
            x = cscale(x, V.rdiag[k + 1 + c0 + i]);
          }
          xi.x = __shfl_sync(0xffffffffu, x.x, i);
          xi.y = __shfl_sync(0xffffffffu, x.y, i);
          if (lane > i && lane < cm) {
            const double2 l = B[(k + 1 + c0 + lane) + (int64_t)(k + 1 + c0 + i) * ldb];
            x.x = fma(-xi.x, l.x, x.x);
            x.x = fma(xi.y, l.y, x.x);
            x.y = fma(-xi.x, l.y, x.y);
            x.y = fma(-xi.y, l.x, x.y);
          }
        }
        if (lane < cm) a[c0 + lane] = x;
      }
      __syncthreads();
      const int rest = m - c0 - cm;
      for (int r = tid; r < rest; r += NT) {
        const int row = c0 + cm + r;
        double2 v = a[row];
        for (int i = 0; i < cm; ++i) {
          const double2 xi = a[c0 + i];
          const double2 l = B[(k + 1 + row) + (int64_t)(k + 1 + c0 + i) * ldb];
          v.x = fma(-xi.x, l.x, v.x);
          v.x = fma(xi.y, l.y, v.x);
          v.y = fma(-xi.x, l.y, v.y);
          v.y = fma(-xi.y, l.x, v.y);
        }
        a[row] = v;
      }
      __syncthreads();
    }
  }
}

// ------------------------------------------------------ tridiagonalisation
__device__ void hetd2_lower(double2* A, int lda, int n, Vecs& V) {
  const int tid = threadIdx.x;
  for (int k = 0; k < n - 1; ++k) {
    const int m = n - k - 1;
    double2* x = A + (k + 1) + (int64_t)k * lda;
    double s = 0.0;
    for (int i = 1 + tid; i < m; i += NT) s = fma(x[i].x, x[i].x, fma(x[i].y, x[i].y, s));
    const double xnorm2 = block_sum(s, V.red);
    if (tid == 0) {
      const double2 alpha = x[0];
      double beta, taur, taui;
      double2 scl = make_double2(0.0, 0.0);
      int trivial = 0;
      if (xnorm2 == 0.0 && alpha.y == 0.0) {
        beta = alpha.x;
        taur = 0.0;
        taui = 0.0;
        trivial = 1;
      } else {
        const double nrm = sqrt(fma(alpha.x, alpha.x, fma(alpha.y, alpha.y, xnorm2)));
        beta = alpha.x >= 0.0 ? -nrm : nrm;
        taur = (beta - alpha.x) / beta;
        taui = -alpha.y / beta;
        // scl = 1 / (alpha - beta)
        const double dr = alpha.x - beta, di = alpha.y;
        const double den = 1.0 / fma(dr, dr, di * di);
        scl = make_double2(dr * den, -di * den);
      }
      V.sc[0] = beta;
      V.sc[1] = taur;
      V.sc[2] = taui;
      V.sc[3] = scl.x;
      V.sc[4] = scl.y;
      reinterpret_cast<int*>(V.sc)[10] = trivial;
      V.d[k] = A[k + (int64_t)k * lda].x;
      V.e2[k] = beta * beta;
    }
    __syncthreads();
    const int trivial = reinterpret_cast<int*>(V.sc)[10];
    const double2 tau = make_double2(V.sc[1], V.sc[2]);
    if (!trivial) {
      const double2 scl = make_double2(V.sc[3], V.sc[4]);
      for (int i = 1 + tid; i < m; i += NT) x[i] = cmul(x[i], scl);
      if (tid == 0) x[0] = make_double2(1.0, 0.0);
      __syncthreads();
      // w = tau * A22 v
      hemv_lower(A, lda, k + 1, m, x, V.w, tau, V.red + 4 * NW);
      // alpha2 = -1/2 tau (w^H v)
      double pr = 0.0, pi = 0.0;
      for (int i = tid; i < m; i += NT) {
        const double2 wi = V.w[i], vi = x[i];
        pr = fma(wi.x, vi.x, fma(wi.y, vi.y, pr));
        pi = fma(wi.x, vi.y, fma(-wi.y, vi.x, pi));
      }
      const double dre = block_sum(pr, V.red);
      const double dim = block_sum(pi, V.red + NW);
      const double2 al = cmul(make_double2(-0.5 * tau.x, -0.5 * tau.y), make_double2(dre, dim));
      for (int i = tid; i < m; i += NT) V.w[i] = cfma(al, x[i], V.w[i]);
      __syncthreads();
      her2_lower(A, lda, k + 1, m, x, 0, V.w);
      __syncthreads();
      if (tid == 0) x[0] = make_double2(V.sc[0], 0.0);
    } else {
      if (tid == 0) {
        A[(k + 1) + (int64_t)(k + 1) * lda].y = 0.0;
      }
    }
    __syncthreads();
  }
  if (tid == 0) V.d[n - 1] = A[(n - 1) + (int64_t)(n - 1) * lda].x;
  __syncthreads();
}

// ------------------------------------------------------- Sturm bisection
// Number of eigenvalues of the tridiagonal (d, e^2) below x.
//
// FP64 count: the determinant recurrence p_i = (d_i - x) p_{i-1} - e_{i-1}^2 p_{i-2}
// (three FP64 operations per step, no division); the count is the number of
// sign changes of p_0..p_n, i.e. of negative pivots q_i = p_i / p_{i-1} of
// the LDL^T factorisation of T - x I.  Signs are read from the bit pattern
// and the pair (p, p_prev) is rescaled by exact powers of two when its
// exponent drifts, so nothing overflows.  An exact zero p_i takes the sign
// opposite to p_{i-1} (the tiny negative pivot LAPACK substitutes).
__device__ __forceinline__ int sign_bit(double v) { return (int)((unsigned long long)__double_as_longlong(v) >> 63); }

__device__ int sturm_count64(const double* d, const double* e2, int n, double x) {
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
    const int ex = (int)((__double_as_longlong(p) >> 52) & 0x7ff);
    if (ex > 1023 + 480 || ex < 1023 - 480) {
      const double f = __longlong_as_double((long long)(2046 - ex) << 52);  // 2^(1023 - ex)
      p *= f;
      pm *= f;
    }
  }
  return c;
}

// FP32 count on the rounded tridiagonal (LDL^T pivots, FP32 division is cheap).
__device__ int sturm_count32(const float* d, const float* e2, int n, float x, float pivmin) {
  float q = d[0] - x;
  int c = q < 0.0f;
  for (int i = 1; i < n; ++i) {
    if (fabsf(q) < pivmin) q = -pivmin;
    q = (d[i] - x) - __fdiv_rn(e2[i - 1], q);
    c += q < 0.0f;
  }
  return c;
}

// Eigenvalue j of the tridiagonal: FP32 bisection brackets it to ~1e-6 of the
// spectrum's scale, two FP64 counts confirm the widened bracket (else the
// full Gershgorin interval is used), and FP64 bisection finishes it to
// 1e-14 of the scale.
__device__ void tridiag_eigenvalues(int n, Vecs& V, double* out) {
  const int tid = threadIdx.x;
  double lo = 1e300, hi = -1e300, emax = 0.0;
  for (int i = tid; i < n; i += NT) {
    const double ea = (i > 0) ? sqrt(V.e2[i - 1]) : 0.0;
    const double eb = (i < n - 1) ? sqrt(V.e2[i]) : 0.0;
    lo = fmin(lo, V.d[i] - ea - eb);
    hi = fmax(hi, V.d[i] + ea + eb);
    if (i < n - 1) emax = fmax(emax, V.e2[i]);
    V.d32[i] = (float)V.d[i];
    V.e232[i] = (float)V.e2[i];
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    emax = fmax(emax, __shfl_xor_sync(0xffffffffu, emax, o));
  }
  __syncthreads();
  if ((tid & 31) == 0) {
    V.red[tid >> 5] = lo;
    V.red[NW + (tid >> 5)] = hi;
    V.red[2 * NW + (tid >> 5)] = emax;
  }
  __syncthreads();
  lo = V.red[0];
  hi = V.red[NW];
  emax = V.red[2 * NW];
  for (int w = 1; w < NW; ++w) {
    lo = fmin(lo, V.red[w]);
    hi = fmax(hi, V.red[NW + w]);
    emax = fmax(emax, V.red[2 * NW + w]);
  }
  const double bnorm = fmax(fmax(fabs(lo), fabs(hi)), 1e-300);
  lo -= 2.2e-16 * bnorm * 4.0 * n + 1e-300;
  hi += 2.2e-16 * bnorm * 4.0 * n + 1e-300;
  const double atol = 1e-14 * bnorm;
  const float pivmin32 = 1.1754944e-38f * fmaxf(1.0f, (float)emax);
  const double margin = 32.0 * 5.9604645e-8 * bnorm;   // covers FP32 rounding of T and of the count
  __syncthreads();
  for (int j = tid; j < n; j += NT) {
    // FP32 bracket
    float a32 = (float)lo, b32 = (float)hi;
    for (int it = 0; it < 40; ++it) {
      const float mid = 0.5f * (a32 + b32);
      if (!(mid > a32 && mid < b32)) break;
      if (sturm_count32(V.d32, V.e232, n, mid, pivmin32) > j) b32 = mid; else a32 = mid;
    }
    double a = (double)a32 - margin, b = (double)b32 + margin;
    if (a < lo) a = lo;
    if (b > hi) b = hi;
    if (!(sturm_count64(V.d, V.e2, n, a) <= j && sturm_count64(V.d, V.e2, n, b) > j)) {
      a = lo;
      b = hi;
    }
    for (int it = 0; it < 200 && (b - a) > atol; ++it) {
      const double mid = 0.5 * (a + b);
      if (mid <= a || mid >= b) break;
      if (sturm_count64(V.d, V.e2, n, mid) > j) b = mid; else a = mid;
    }
    out[j] = 0.5 * (a + b);
  }
}

// Unit diagonal for rows/columns that are entirely zero (eighb's aux option,
// slakonet/utils.py:741-747).  Integer tests only.
__device__ void aux_zero_rows(double2* A, int lda, int n) {
  for (int i = threadIdx.x; i < n; i += NT) {
    bool zero = true;
    for (int j = 0; j < n && zero; ++j) {
      const double2 v = (j <= i) ? A[i + (int64_t)j * lda] : A[j + (int64_t)i * lda];
      zero = is_zero_bits(v.x) && is_zero_bits(v.y);
    }
    if (zero) A[i + (int64_t)i * lda].x += 1.0;
  }
}

__global__ void __launch_bounds__(NT) k_eigh_gen(int n_prob, const int32_t* __restrict__ nvec,
                                                 const int64_t* __restrict__ hs_off,
                                                 const int64_t* __restrict__ eig_off,
                                                 const int32_t* __restrict__ order, double2* H, double2* S,
                                                 double* __restrict__ eig, int32_t* __restrict__ status,
                                                 int32_t* __restrict__ counter, int max_n, int use_smem_mats) {
  extern __shared__ double smem[];
  const int tid = threadIdx.x;
  Vecs V;
  {
    double* p = smem;
    V.sc = p; p += 16;
    V.red = p; p += 4 * NW + 2 * NT;
    V.d = p; p += max_n;
    V.e2 = p; p += max_n;
    V.rdiag = p; p += max_n;
    p += (max_n & 1);
    V.w = reinterpret_cast<double2*>(p); p += 2 * max_n;
    V.d32 = reinterpret_cast<float*>(V.rdiag);
    V.e232 = V.d32 + max_n;
  }
  double2* Hs = reinterpret_cast<double2*>(smem + 16 + 4 * NW + 2 * NT + 3 * max_n + (max_n & 1) + 2 * max_n);
  double2* Ss = Hs + SMEM_LDA * SMEM_N;
  __shared__ int s_idx;
  for (;;) {
    if (tid == 0) s_idx = atomicAdd(counter, 1);
    __syncthreads();
    const int idx = s_idx;
    __syncthreads();
    if (idx >= n_prob) break;
    const int p = order[idx];
    const int n = nvec[p];
    double2* Hg = H + hs_off[p];
    double2* Sg = S + hs_off[p];
    double2 *Ha, *Sa;
    int lda;
    const bool in_smem = use_smem_mats && n <= SMEM_N;
    if (in_smem) {
      lda = SMEM_LDA;
      Ha = Hs;
      Sa = Ss;
      for (int e = tid; e < n * n; e += NT) {
        const int i = e % n, j = e / n;
        if (i >= j) {
          Ha[i + j * lda] = Hg[e];
          Sa[i + j * lda] = Sg[e];
        }
      }
    } else {
      lda = n;
      Ha = Hg;
      Sa = Sg;
    }
    __syncthreads();
    aux_zero_rows(Ha, lda, n);
    aux_zero_rows(Sa, lda, n);
    __syncthreads();
    const bool ok = cholesky_lower(Sa, lda, n, V);
    if (!ok) {
      for (int j = tid; j < n; j += NT) eig[eig_off[p] + j] = __longlong_as_double(0x7ff8000000000000LL);
      if (tid == 0) status[p] = SKN_ERR_NOT_SPD;
      __syncthreads();
      continue;
    }
    hegs2_lower(Ha, lda, Sa, lda, n, V);
    hetd2_lower(Ha, lda, n, V);
    if (n == 1 && tid == 0) V.d[0] = Ha[0].x;
    __syncthreads();
    tridiag_eigenvalues(n, V, eig + eig_off[p]);
    if (tid == 0) status[p] = SKN_OK;
    __syncthreads();
  }
}

}  // namespace

extern "C" int skn_eigh_gen_batched(int n_prob, const int32_t* n, const int64_t* hs_off, const int64_t* eig_off,
                                    const int32_t* order, double* H, double* S, double* eig, int32_t* status,
                                    int32_t* work_counter, int max_n, cudaStream_t stream) {
  if (n_prob < 0 || max_n < 0) return SKN_ERR_ARG;
  if (n_prob == 0) return SKN_OK;
  if (!n || !hs_off || !eig_off || !order || !H || !S || !eig || !status || !work_counter) return SKN_ERR_ARG;
  if (max_n > MAX_N) return SKN_ERR_CAPACITY;
  const int mn = max_n < 1 ? 1 : max_n;
  const int use_smem_mats = 1;
  size_t smem = sizeof(double) * (16 + 4 * NW + 2 * NT + 3 * (size_t)mn + (mn & 1) + 2 * (size_t)mn);
  smem += (size_t)use_smem_mats * 2 * SMEM_LDA * SMEM_N * sizeof(double2);
  if (cudaFuncSetAttribute(k_eigh_gen, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return SKN_ERR_CUDA;
  int per_sm = 0, dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_eigh_gen, NT, smem) != cudaSuccess || per_sm < 1)
    return SKN_ERR_CUDA;
  int grid = sms * per_sm;
  if (grid > n_prob) grid = n_prob;
  if (cudaMemsetAsync(work_counter, 0, sizeof(int32_t), stream) != cudaSuccess) return SKN_ERR_CUDA;
  k_eigh_gen<<<grid, NT, smem, stream>>>(n_prob, n, hs_off, eig_off, order, (double2*)H, (double2*)S, eig, status,
                                         work_counter, mn, use_smem_mats);
  return cudaPeekAtLastError() == cudaSuccess ? SKN_OK : SKN_ERR_CUDA;
}
