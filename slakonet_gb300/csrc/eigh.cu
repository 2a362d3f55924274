// Batched generalized Hermitian eigenvalues, FP64, one CTA per problem.
//
// For each (structure, k) problem H x = e S x the CTA runs
//   1. Cholesky S = L L^H (lower, right-looking, in place),
//   2. reduction to C = L^-1 H L^-H (LAPACK zhegs2 order: scale, axpy,
//      her2, axpy, triangular solve per column),
//   3. Householder tridiagonalisation of C (zhetd2: larfg, hemv, her2),
//   4. eigenvalues of the real tridiagonal from Sturm counts (FP32 bracket,
//      then FP64 Newton on the characteristic polynomial for isolated
//      eigenvalues, FP64 bisection for clusters), one thread per eigenvalue,
//      which returns them in ascending order.
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
#include "sturm.cuh"

// Exported names carry SKN_EIG_SUFFIX so several launch shapes can live in one library.
#ifndef SKN_EIG_SUFFIX
#define SKN_EIG_SUFFIX
#endif
#define SKN_CAT2(a, b) a##b
#define SKN_CAT(a, b) SKN_CAT2(a, b)
#define SKN_EXPORT(name) SKN_CAT(name, SKN_EIG_SUFFIX)
// Every compiled copy of this file keeps its kernels in its own namespace, so the
// copies (launch shapes, and files that include this one) link side by side.
#ifndef SKN_EIG_NS_TAG
#define SKN_EIG_NS_TAG SKN_EIG_SUFFIX
#endif
#define SKN_EIG_NS SKN_CAT(skn_eig, SKN_EIG_NS_TAG)

namespace SKN_EIG_NS {
namespace {

// Launch shape knobs (compile-time; tuned by the size sweep):
#ifndef SKN_EIG_NT
#define SKN_EIG_NT 128
#endif
#ifndef SKN_EIG_MINB
#define SKN_EIG_MINB 5
#endif
#ifndef SKN_EIG_UNR
#define SKN_EIG_UNR 2
#endif
#ifndef SKN_EIG_SMEM_N
#define SKN_EIG_SMEM_N 24
#endif
constexpr int NT = SKN_EIG_NT;    // threads per CTA
constexpr int NW = NT / 32;
constexpr int SMEM_N = SKN_EIG_SMEM_N;   // problems up to this size run from shared memory
constexpr int SMEM_LDA = SMEM_N + 1;
// The shared-memory region stages small problems (H and S, 2*SMEM_LDA*SMEM_N elements) and,
// for problems solved in global memory, holds the 32x33 tile of the triangular solve.
constexpr int TILE_ELEMS = 32 * 33;
constexpr int SMEM_REGION = (2 * SMEM_LDA * SMEM_N > TILE_ELEMS) ? 2 * SMEM_LDA * SMEM_N : TILE_ELEMS;
static_assert(SMEM_REGION >= TILE_ELEMS && SMEM_REGION >= 2 * SMEM_LDA * SMEM_N, "staging region too small");
constexpr int MAX_N = 2048;       // shared-memory vectors bound the single-CTA path

struct Vecs {
  double2* v;      // n: working column / Householder vector
  double2* w;      // n: hemv result / Householder w / L column
  double* d;       // n: tridiagonal diagonal
  double* e2;      // n: squared off-diagonal (e2[i] couples i and i+1)
  double* rdiag;   // n: 1 / L[i][i]
  double* red;     // 4 * NW reduction scratch
  double* sc;      // 16 scalars
  float* d32;      // n: FP32 copy of d (aliases rdiag, free after the reduction)
  float* e232;     // n: FP32 copy of e^2
};

// c - conj(a) * b
__device__ __forceinline__ double2 cfms_conj_l(double2 a, double2 b, double2 c) {
  c.x = fma(-a.x, b.x, c.x);
  c.x = fma(-a.y, b.y, c.x);
  c.y = fma(-a.x, b.y, c.y);
  c.y = fma(a.y, b.x, c.y);
  return c;
}

// Arithmetic on complex entries, or on their real parts alone when the problem
// is real (R = true: every imaginary part of H and S is exactly zero, as at
// k-points with 2k integer, where the Bloch phases are exactly +-1).  With R
// the imaginary parts are never loaded, computed or stored; each real part
// comes out of the same fused operations as in the complex code, minus terms
// that are exactly zero, so both paths give the same numbers on a real problem
// while the real one issues a quarter of the FP64 instructions.
template <bool R> SKN_DEVINL double2 z_ld(const double2* p) {
  if constexpr (R) return make_double2(p->x, 0.0); else return *p;
}
template <bool R> SKN_DEVINL void z_st(double2* p, double2 v) {
  if constexpr (R) p->x = v.x; else *p = v;
}
template <bool R> SKN_DEVINL double2 z_fma(double2 a, double2 b, double2 c) {   // c + a b
  if constexpr (R) { c.x = fma(a.x, b.x, c.x); return c; } else return cfma(a, b, c);
}
template <bool R> SKN_DEVINL double2 z_fms_conj(double2 a, double2 b, double2 c) {   // c - a conj(b)
  if constexpr (R) { c.x = fma(-a.x, b.x, c.x); return c; } else return cfms_conj(a, b, c);
}
template <bool R> SKN_DEVINL double2 z_mul(double2 a, double2 b) {
  if constexpr (R) return make_double2(a.x * b.x, 0.0); else return cmul(a, b);
}
template <bool R> SKN_DEVINL double2 z_scale(double2 a, double s) {
  if constexpr (R) return make_double2(a.x * s, 0.0); else return cscale(a, s);
}
template <bool R> SKN_DEVINL double2 z_axpy(double a, double2 x, double2 y) {   // y + a x, a real
  y.x = fma(a, x.x, y.x);
  if constexpr (!R) y.y = fma(a, x.y, y.y);
  return y;
}
template <bool R> SKN_DEVINL double2 z_sub_mul(double2 v, double2 x, double2 l) {   // v - x l
  v.x = fma(-x.x, l.x, v.x);
  if constexpr (!R) {
    v.x = fma(x.y, l.y, v.x);
    v.y = fma(-x.x, l.y, v.y);
    v.y = fma(-x.y, l.x, v.y);
  }
  return v;
}

// ---------------------------------------------------------------- Cholesky
// Loops over the trailing triangle issue UNR independent loads per thread
// before their FMAs: with FP64 this slow, the kernel is bound by how many
// global loads each SM keeps in flight, not by bandwidth.
constexpr int UNR = SKN_EIG_UNR;
static_assert(UNR >= 2 && UNR % 2 == 0, "unrolled loops pair their accumulators");

template <bool R>
__device__ bool cholesky_lower(double2* __restrict__ A, int lda, int n, Vecs& V) {
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
    double2* col = A + (k + 1) + (int64_t)k * lda;
    for (int i = tid; i < m; i += NT) {
      const double2 v = z_scale<R>(z_ld<R>(col + i), rd);
      z_st<R>(col + i, v);
      V.v[i] = v;
    }
    __syncthreads();
    // trailing update of the packed lower triangle (k < j <= i): A_ij -= l_i conj(l_j)
    const int tri = m * (m + 1) / 2;
    double2* T = A + (k + 1) + (int64_t)(k + 1) * lda;
    for (int e0 = tid; e0 < tri; e0 += NT * UNR) {
      int off[UNR], ii[UNR], jj[UNR];
      double2 a[UNR];
#pragma unroll
      for (int u = 0; u < UNR; ++u) {
        const int e = e0 + u * NT;
        if (e < tri) {
          tri_index(e, m, ii[u], jj[u]);
          off[u] = ii[u] + jj[u] * lda;
          a[u] = z_ld<R>(T + off[u]);
        }
      }
#pragma unroll
      for (int u = 0; u < UNR; ++u) {
        if (e0 + u * NT < tri) z_st<R>(T + off[u], z_fms_conj<R>(V.v[ii[u]], V.v[jj[u]], a[u]));
      }
    }
    __syncthreads();
  }
  return true;
}

// y[i] = scale * sum_j Herm(A22)[i][j] x[j] for i < m, A22 at A (lower stored),
// x in shared memory.  Rows on lanes with a uniform trip count over j, UNR
// loads in flight per thread.  Full passes take NT rows; the remaining
// m mod NT rows (all rows when m < NT) go to as many warps as they fill, and
// when that leaves warps over, the warps split the j range and partial sums
// are combined through `part`.  No thread computes a row twice, so a warp
// issues FP64 work only for rows that exist.
template <bool R>
__device__ __forceinline__ double2 hemv_row(const double2* __restrict__ A, int lda, int i, int j0, int j1,
                                            const double2* __restrict__ x) {
  double2 acc0 = make_double2(0.0, 0.0), acc1 = make_double2(0.0, 0.0);
  int j = j0;
  for (; j + UNR <= j1; j += UNR) {
    double2 a[UNR];
#pragma unroll
    for (int u = 0; u < UNR; ++u) {
      const int jj = j + u;
      const bool up = jj > i;
      a[u] = z_ld<R>(up ? A + jj + (int64_t)i * lda : A + i + (int64_t)jj * lda);
      if constexpr (!R) a[u].y = cond_flip(a[u].y, up);
    }
#pragma unroll
    for (int u = 0; u < UNR; u += 2) {
      acc0 = z_fma<R>(a[u], x[j + u], acc0);
      acc1 = z_fma<R>(a[u + 1], x[j + u + 1], acc1);
    }
  }
  for (; j < j1; ++j) {
    const bool up = j > i;
    double2 a = z_ld<R>(up ? A + j + (int64_t)i * lda : A + i + (int64_t)j * lda);
    if constexpr (!R) a.y = cond_flip(a.y, up);
    acc0 = z_fma<R>(a, x[j], acc0);
  }
  return make_double2(acc0.x + acc1.x, acc0.y + acc1.y);
}

template <bool R>
__device__ void hemv_lower(const double2* __restrict__ A, int lda, int m, const double2* __restrict__ x,
                           double2* __restrict__ y, double2 scale, double2* __restrict__ part) {
  const int tid = threadIdx.x;
  const int full = (m / NT) * NT;
  for (int rbase = 0; rbase < full; rbase += NT) y[rbase + tid] = z_mul<R>(scale, hemv_row<R>(A, lda, rbase + tid, 0, m, x));
  const int rem = m - full;
  if (rem > 0) {
    const int row_warps = (rem + 31) >> 5;            // <= NW
    const int nsplit = NW / row_warps;
    const int w = tid >> 5, lane = tid & 31;
    const int sp = w / row_warps;
    const int r_in = (w % row_warps) * 32 + lane;
    const int i = full + min(r_in, rem - 1);
    const int chunk = (m + nsplit - 1) / nsplit;
    const int j0 = sp * chunk, j1 = min(m, j0 + chunk);
    double2 acc = make_double2(0.0, 0.0);
    if (sp < nsplit) acc = hemv_row<R>(A, lda, i, j0, j1, x);
    if (nsplit == 1) {
      if (sp == 0 && r_in < rem) y[full + r_in] = z_mul<R>(scale, acc);
    } else {
      part[tid] = acc;
      __syncthreads();
      for (int r = tid; r < rem; r += NT) {
        double2 s = make_double2(0.0, 0.0);
        const int rbw = r >> 5, ln = r & 31;
        for (int q = 0; q < nsplit; ++q) {
          const double2 v = part[(q * row_warps + rbw) * 32 + ln];
          s.x += v.x;
          s.y += v.y;
        }
        y[full + r] = z_mul<R>(scale, s);
      }
    }
  }
  __syncthreads();
}

// A22 -= x y^H + y x^H on the packed lower triangle (A22 at T), x and y in shared memory.
template <bool R>
__device__ void her2_lower(double2* __restrict__ T, int lda, int m, const double2* __restrict__ x,
                           const double2* __restrict__ y) {
  const int tri = m * (m + 1) / 2;
  for (int e0 = threadIdx.x; e0 < tri; e0 += NT * UNR) {
    int off[UNR], ii[UNR], jj[UNR];
    double2 a[UNR];
#pragma unroll
    for (int u = 0; u < UNR; ++u) {
      const int e = e0 + u * NT;
      if (e < tri) {
        tri_index(e, m, ii[u], jj[u]);
        off[u] = ii[u] + jj[u] * lda;
        a[u] = z_ld<R>(T + off[u]);
      }
    }
#pragma unroll
    for (int u = 0; u < UNR; ++u) {
      if (e0 + u * NT < tri) {
        double2 v = z_fms_conj<R>(x[ii[u]], y[jj[u]], a[u]);
        z_st<R>(T + off[u], z_fms_conj<R>(y[ii[u]], x[jj[u]], v));
      }
    }
  }
}

// ------------------------------------------------- reduction to standard form
// A (lower) <- L^-1 A L^-H with B = L from cholesky_lower (rdiag holds 1/L_kk),
// column by column in LAPACK zhegs2 order.  The working column and the L
// column live in shared memory for the rank-2 update and the solve.
template <bool R>
__device__ void hegs2_lower(double2* __restrict__ A, int lda, const double2* __restrict__ B, int ldb, int n,
                            Vecs& V, double2* tile) {
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
    double2* acol = A + (k + 1) + (int64_t)k * lda;
    const double2* bcol = B + (k + 1) + (int64_t)k * ldb;
    double2* a = V.v;
    double2* b = V.w;
    for (int i = tid; i < m; i += NT) {
      const double2 bi = z_ld<R>(bcol + i);
      a[i] = z_axpy<R>(ct, bi, z_scale<R>(z_ld<R>(acol + i), rd));
      b[i] = bi;
    }
    __syncthreads();
    her2_lower<R>(A + (k + 1) + (int64_t)(k + 1) * lda, lda, m, a, b);
    __syncthreads();   // the update above reads a[]; the axpy below rewrites it
    for (int i = tid; i < m; i += NT) {
      a[i] = z_axpy<R>(ct, b[i], a[i]);
    }
    __syncthreads();
    // forward substitution a <- L22^-1 a in chunks of 32 rows: warp 0 solves the
    // diagonal chunk, then all threads apply it to the rows below.
    const double2* L = B + (k + 1) + (int64_t)(k + 1) * ldb;
    for (int c0 = 0; c0 < m; c0 += 32) {
      const int cm = min(32, m - c0);
      // stage the cm x cm diagonal block of L (from global memory) in the tile
      const double2* Ld = L + c0 + (int64_t)c0 * ldb;
      int ldt = ldb;
      if (tile != nullptr) {
        for (int e = tid; e < cm * 32; e += NT) {
          const int r = e & 31, c = e >> 5;
          if (r < cm) tile[r + c * 33] = z_ld<R>(Ld + r + (int64_t)c * ldb);
        }
        __syncthreads();
        Ld = tile;
        ldt = 33;
      }
      if (tid < 32) {
        const int lane = tid;
        double2 xv = (lane < cm) ? a[c0 + lane] : make_double2(0.0, 0.0);
        for (int i = 0; i < cm; ++i) {
          if (lane == i) xv = z_scale<R>(xv, V.rdiag[k + 1 + c0 + i]);
          double2 xi;
          xi.x = __shfl_sync(0xffffffffu, xv.x, i);
          xi.y = R ? 0.0 : __shfl_sync(0xffffffffu, xv.y, i);
          if (lane > i && lane < cm) {
            xv = z_sub_mul<R>(xv, xi, z_ld<R>(Ld + lane + (int64_t)i * ldt));
          }
        }
        if (lane < cm) a[c0 + lane] = xv;
      }
      __syncthreads();
      const int rest = m - c0 - cm;
      for (int r = tid; r < rest; r += NT) {
        const int row = c0 + cm + r;
        double2 v0 = a[row], v1 = make_double2(0.0, 0.0);
        const double2* Lr = L + row + (int64_t)c0 * ldb;
        int i = 0;
        for (; i + UNR <= cm; i += UNR) {
          double2 l[UNR];
#pragma unroll
          for (int u = 0; u < UNR; ++u) l[u] = z_ld<R>(Lr + (int64_t)(i + u) * ldb);
#pragma unroll
          for (int u = 0; u < UNR; u += 2) {
            v0 = z_sub_mul<R>(v0, a[c0 + i + u], l[u]);
            v1 = z_sub_mul<R>(v1, a[c0 + i + u + 1], l[u + 1]);
          }
        }
        for (; i < cm; ++i) {
          v0 = z_sub_mul<R>(v0, a[c0 + i], z_ld<R>(Lr + (int64_t)i * ldb));
        }
        a[row] = make_double2(v0.x + v1.x, v0.y + v1.y);
      }
      __syncthreads();
    }
    for (int i = tid; i < m; i += NT) z_st<R>(acol + i, a[i]);
    __syncthreads();
  }
}

// ------------------------------------- blocked Cholesky and reduction (NB-column panels)
// The same factorisations in LAPACK's blocked order (zpotrf right-looking, zhegst itype 1,
// lower).  Per panel: a small unblocked step on the NB x NB diagonal block in shared memory,
// row-parallel triangular solves of the panel, then one trailing update of the packed lower
// triangle in which every element accumulates all NB panel terms in registers -- one
// read-modify-write per element per panel instead of per column, full warps on contiguous
// elements, and one barrier per phase instead of several per column.
#ifndef SKN_EIG_BLOCKED
#define SKN_EIG_BLOCKED 0
#endif
constexpr int NB = 32;          // panel width
constexpr int LDT = NB + 1;     // leading dimension of the shared-memory tiles
static_assert(SMEM_REGION >= NB * LDT, "the staging region doubles as the first panel tile");

// c - sum_k P[i,k] conj(Q[j,k]) over the NB columns of two panels (column strides lp, lq), two chains.
template <bool R>
SKN_DEVINL double2 panel_dot_conj(const double2* __restrict__ Pi, int lp, const double2* __restrict__ Qj, int lq,
                                  double2 c) {
  double2 acc1 = make_double2(0.0, 0.0);
#pragma unroll 8
  for (int k = 0; k < NB; k += 2) {
    c = z_fms_conj<R>(z_ld<R>(Pi + (int64_t)k * lp), z_ld<R>(Qj + (int64_t)k * lq), c);
    acc1 = z_fms_conj<R>(z_ld<R>(Pi + (int64_t)(k + 1) * lp), z_ld<R>(Qj + (int64_t)(k + 1) * lq), acc1);
  }
  return make_double2(c.x + acc1.x, c.y + acc1.y);
}

// x L^H = a for the w entries of one row (stride ld), L lower w x w in the shared tile Lt,
// rd[j] = 1 / L_jj; in place.  Entries already solved are re-read from memory (same thread).
template <bool R>
SKN_DEVINL void row_solve_lh(double2* __restrict__ row, int64_t ld, const double2* __restrict__ Lt, int w,
                             const double* __restrict__ rd) {
  for (int j = 0; j < w; ++j) {
    double2 a0 = z_ld<R>(row + j * ld), a1 = make_double2(0.0, 0.0);
    int k = 0;
    for (; k + 1 < j; k += 2) {
      a0 = z_fms_conj<R>(z_ld<R>(row + k * ld), Lt[j + k * LDT], a0);
      a1 = z_fms_conj<R>(z_ld<R>(row + (k + 1) * ld), Lt[j + (k + 1) * LDT], a1);
    }
    if (k < j) a0 = z_fms_conj<R>(z_ld<R>(row + k * ld), Lt[j + k * LDT], a0);
    z_st<R>(row + j * ld, z_scale<R>(make_double2(a0.x + a1.x, a0.y + a1.y), rd[j]));
  }
}

// S = L L^H in place (lower), panels of NB columns; V.rdiag[k] = 1 / L_kk.  Lt: NB x LDT tile.
// Returns false (every thread) when S is not positive definite.
template <bool R>
__device__ bool cholesky_blocked(double2* __restrict__ A, int lda, int n, Vecs& V, double2* __restrict__ Lt) {
  const int tid = threadIdx.x;
  int* flag = reinterpret_cast<int*>(V.sc) + 2;
  for (int c0 = 0; c0 < n; c0 += NB) {
    const int w = min(NB, n - c0);
    const int m = n - c0 - w;
    double2* A11 = A + c0 + (int64_t)c0 * lda;
    for (int e = tid; e < w * w; e += NT) {
      const int i = e % w, j = e / w;
      if (i >= j) Lt[i + j * LDT] = z_ld<R>(A11 + i + (int64_t)j * lda);
    }
    __syncthreads();
    if (tid < 32) {             // unblocked Cholesky of the diagonal block, lane = row
      const int lane = tid;
      int bad = 0;
      for (int k = 0; k < w; ++k) {
        const double a = Lt[k + k * LDT].x;
        const bool ok = (a > 0.0) && is_finite_bits(a);
        bad |= ok ? 0 : 1;
        const double dk = ok ? sqrt(a) : 1.0;
        const double rd = 1.0 / dk;
        __syncwarp();
        if (lane == k) {
          Lt[k + k * LDT] = make_double2(dk, 0.0);
          V.rdiag[c0 + k] = rd;
        }
        double2 lik = make_double2(0.0, 0.0);
        if (lane > k && lane < w) {
          lik = z_scale<R>(Lt[lane + k * LDT], rd);
          Lt[lane + k * LDT] = lik;
        }
        __syncwarp();
        if (lane > k && lane < w)
          for (int j = k + 1; j <= lane; ++j) Lt[lane + j * LDT] = z_fms_conj<R>(lik, Lt[j + k * LDT], Lt[lane + j * LDT]);
        __syncwarp();
      }
      if (lane == 0) *flag = bad;
    }
    __syncthreads();
    if (*flag) return false;
    for (int e = tid; e < w * w; e += NT) {
      const int i = e % w, j = e / w;
      if (i >= j) z_st<R>(A11 + i + (int64_t)j * lda, Lt[i + j * LDT]);
    }
    if (m > 0) {                // here w == NB
      double2* A21 = A11 + w;
      for (int r = tid; r < m; r += NT) row_solve_lh<R>(A21 + r, lda, Lt, NB, V.rdiag + c0);
      __syncthreads();
      double2* A22 = A21 + (int64_t)w * lda;
      const int tri = m * (m + 1) / 2;
      for (int e = tid; e < tri; e += NT) {
        int i, j;
        tri_index(e, m, i, j);
        double2* t = A22 + i + (int64_t)j * lda;
        z_st<R>(t, panel_dot_conj<R>(A21 + i, lda, A21 + j, lda, z_ld<R>(t)));
      }
    }
    __syncthreads();
  }
  return true;
}

// A21 -= 1/2 L21 A11 for the m x NB panel, A11 Hermitian (both triangles) in the tile At.
template <bool R>
__device__ void panel_hemm_half(double2* __restrict__ A21, int lda, const double2* __restrict__ L21, int ldb, int m,
                                const double2* __restrict__ At) {
  for (int e = threadIdx.x; e < m * NB; e += NT) {
    const int r = e % m, j = e / m;
    double2 s0 = make_double2(0.0, 0.0), s1 = s0;
#pragma unroll 8
    for (int k = 0; k < NB; k += 2) {
      s0 = z_fma<R>(z_ld<R>(L21 + r + (int64_t)k * ldb), At[k + j * LDT], s0);
      s1 = z_fma<R>(z_ld<R>(L21 + r + (int64_t)(k + 1) * ldb), At[k + 1 + j * LDT], s1);
    }
    double2* t = A21 + r + (int64_t)j * lda;
    z_st<R>(t, z_axpy<R>(-0.5, make_double2(s0.x + s1.x, s0.y + s1.y), z_ld<R>(t)));
  }
}

// A (lower) <- L^-1 A L^-H with B = L from cholesky_blocked, LAPACK zhegst order per panel:
// zhegs2 on the diagonal block, A21 L11^-H, -1/2 L21 A11, her2k A22 -= A21 L21^H + L21 A21^H,
// -1/2 L21 A11, L22^-1 A21 (32-row chunks: a one-warp solve of the chunk, lanes over the NB
// right-hand sides, then all threads update the rows below).  Lt, At: NB x LDT tiles.
template <bool R>
__device__ void hegst_blocked(double2* __restrict__ A, int lda, const double2* __restrict__ B, int ldb, int n,
                              Vecs& V, double2* __restrict__ Lt, double2* __restrict__ At) {
  const int tid = threadIdx.x;
  for (int c0 = 0; c0 < n; c0 += NB) {
    const int w = min(NB, n - c0);
    const int m = n - c0 - w;
    double2* A11 = A + c0 + (int64_t)c0 * lda;
    const double2* L11 = B + c0 + (int64_t)c0 * ldb;
    for (int e = tid; e < w * w; e += NT) {
      const int i = e % w, j = e / w;
      if (i >= j) {
        Lt[i + j * LDT] = z_ld<R>(L11 + i + (int64_t)j * ldb);
        At[i + j * LDT] = z_ld<R>(A11 + i + (int64_t)j * lda);
      }
    }
    __syncthreads();
    {
      Vecs Vb = V;
      Vb.rdiag = V.rdiag + c0;
      hegs2_lower<R>(At, LDT, Lt, LDT, w, Vb, nullptr);   // ends with a barrier
    }
    for (int e = tid; e < w * w; e += NT) {
      const int i = e % w, j = e / w;
      if (i >= j) z_st<R>(A11 + i + (int64_t)j * lda, At[i + j * LDT]);
    }
    if (m == 0) break;
    __syncthreads();
    for (int e = tid; e < w * w; e += NT) {     // the reduced block as a full Hermitian tile
      const int i = e % w, j = e / w;
      if (i > j) {
        const double2 v = At[i + j * LDT];
        At[j + i * LDT] = make_double2(v.x, R ? 0.0 : -v.y);
      }
    }
    double2* A21 = A11 + w;
    const double2* L21 = L11 + w;
    for (int r = tid; r < m; r += NT) row_solve_lh<R>(A21 + r, lda, Lt, NB, V.rdiag + c0);
    __syncthreads();
    panel_hemm_half<R>(A21, lda, L21, ldb, m, At);
    __syncthreads();
    double2* A22 = A21 + (int64_t)w * lda;
    const int tri = m * (m + 1) / 2;
    for (int e = tid; e < tri; e += NT) {
      int i, j;
      tri_index(e, m, i, j);
      double2* t = A22 + i + (int64_t)j * lda;
      double2 c = panel_dot_conj<R>(A21 + i, lda, L21 + j, ldb, z_ld<R>(t));
      c = panel_dot_conj<R>(L21 + i, ldb, A21 + j, lda, c);
      z_st<R>(t, c);
    }
    __syncthreads();
    panel_hemm_half<R>(A21, lda, L21, ldb, m, At);
    __syncthreads();
    // A21 <- L22^-1 A21
    const double2* L22 = L21 + (int64_t)w * ldb;
    for (int r0 = 0; r0 < m; r0 += 32) {
      const int cm = min(32, m - r0);
      for (int e = tid; e < cm * cm; e += NT) {
        const int i = e % cm, j = e / cm;
        if (i >= j) Lt[i + j * LDT] = z_ld<R>(L22 + (r0 + i) + (int64_t)(r0 + j) * ldb);
      }
      for (int e = tid; e < cm * NB; e += NT) {
        const int i = e % cm, j = e / cm;
        At[i + j * LDT] = z_ld<R>(A21 + (r0 + i) + (int64_t)j * lda);
      }
      __syncthreads();
      if (tid < NB) {
        const int j = tid;
        const double* rd = V.rdiag + c0 + w + r0;
        for (int i = 0; i < cm; ++i) {
          double2 a0 = At[i + j * LDT], a1 = make_double2(0.0, 0.0);
          int q = 0;
          for (; q + 1 < i; q += 2) {
            a0 = z_sub_mul<R>(a0, Lt[i + q * LDT], At[q + j * LDT]);
            a1 = z_sub_mul<R>(a1, Lt[i + (q + 1) * LDT], At[q + 1 + j * LDT]);
          }
          if (q < i) a0 = z_sub_mul<R>(a0, Lt[i + q * LDT], At[q + j * LDT]);
          At[i + j * LDT] = z_scale<R>(make_double2(a0.x + a1.x, a0.y + a1.y), rd[i]);
        }
      }
      __syncthreads();
      for (int e = tid; e < cm * NB; e += NT) {
        const int i = e % cm, j = e / cm;
        z_st<R>(A21 + (r0 + i) + (int64_t)j * lda, At[i + j * LDT]);
      }
      const int rest = m - r0 - cm;
      for (int e = tid; e < rest * NB; e += NT) {
        const int r = e % rest, j = e / rest;
        const double2* Lr = L22 + (r0 + cm + r) + (int64_t)r0 * ldb;
        double2* t = A21 + (r0 + cm + r) + (int64_t)j * lda;
        double2 a0 = z_ld<R>(t), a1 = make_double2(0.0, 0.0);
        int q = 0;
        for (; q + 1 < cm; q += 2) {
          a0 = z_sub_mul<R>(a0, At[q + j * LDT], z_ld<R>(Lr + (int64_t)q * ldb));
          a1 = z_sub_mul<R>(a1, At[q + 1 + j * LDT], z_ld<R>(Lr + (int64_t)(q + 1) * ldb));
        }
        if (q < cm) a0 = z_sub_mul<R>(a0, At[q + j * LDT], z_ld<R>(Lr + (int64_t)q * ldb));
        z_st<R>(t, make_double2(a0.x + a1.x, a0.y + a1.y));
      }
      __syncthreads();
    }
  }
  __syncthreads();
}

// ------------------------------------------------------ tridiagonalisation
// LAPACK zhetd2 (lower): reflector from column k, w = tau A22 v,
// w -= (tau/2)(w^H v) v, A22 -= v w^H + w v^H.  d and e^2 go to shared memory.
template <bool R>
__device__ void hetd2_lower(double2* __restrict__ A, int lda, int n, Vecs& V, double* tri) {
  const int tid = threadIdx.x;
  for (int k = 0; k < n - 1; ++k) {
    const int m = n - k - 1;
    double2* x = A + (k + 1) + (int64_t)k * lda;
    double s = 0.0;
    for (int i = 1 + tid; i < m; i += NT) {
      const double2 xi = z_ld<R>(x + i);
      V.v[i] = xi;
      s = R ? fma(xi.x, xi.x, s) : fma(xi.x, xi.x, fma(xi.y, xi.y, s));
    }
    const double xnorm2 = block_sum(s, V.red);
    if (tid == 0) {
      const double2 alpha = z_ld<R>(x);
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
      if (tri != nullptr) {          // e (signed) and tau for the eigenvector back-transformation
        tri[n + k] = beta;
        tri[2 * n + 2 * k] = taur;
        tri[2 * n + 2 * k + 1] = taui;
      }
      V.v[0] = make_double2(1.0, 0.0);
    }
    __syncthreads();
    const int trivial = reinterpret_cast<int*>(V.sc)[10];
    const double2 tau = make_double2(V.sc[1], V.sc[2]);
    if (!trivial) {
      const double2 scl = make_double2(V.sc[3], V.sc[4]);
      for (int i = 1 + tid; i < m; i += NT) {
        const double2 v = z_mul<R>(V.v[i], scl);
        V.v[i] = v;
        z_st<R>(x + i, v);
      }
      __syncthreads();
      double2* T = A + (k + 1) + (int64_t)(k + 1) * lda;
      hemv_lower<R>(T, lda, m, V.v, V.w, tau, reinterpret_cast<double2*>(V.red + 4 * NW));
      double pr = 0.0, pi = 0.0;
      for (int i = tid; i < m; i += NT) {
        const double2 wi = V.w[i], vi = V.v[i];
        if constexpr (R) {
          pr = fma(wi.x, vi.x, pr);
        } else {
          pr = fma(wi.x, vi.x, fma(wi.y, vi.y, pr));
          pi = fma(wi.x, vi.y, fma(-wi.y, vi.x, pi));
        }
      }
      const double dre = block_sum(pr, V.red);
      const double dim = R ? 0.0 : block_sum(pi, V.red + NW);
      const double2 al = z_mul<R>(make_double2(-0.5 * tau.x, -0.5 * tau.y), make_double2(dre, dim));
      for (int i = tid; i < m; i += NT) V.w[i] = z_fma<R>(al, V.v[i], V.w[i]);
      __syncthreads();
      her2_lower<R>(T, lda, m, V.v, V.w);
      __syncthreads();
      if (tid == 0) x[0] = make_double2(V.sc[0], 0.0);
    } else {
      if (tid == 0) A[(k + 1) + (int64_t)(k + 1) * lda].y = 0.0;
    }
    __syncthreads();
  }
  if (tid == 0) V.d[n - 1] = A[(n - 1) + (int64_t)(n - 1) * lda].x;
  __syncthreads();
  if (tri != nullptr) {
    for (int i = tid; i < n; i += NT) tri[i] = V.d[i];
    if (tid == 0) {
      tri[2 * n - 1] = 0.0;
      tri[4 * n - 2] = 0.0;
      tri[4 * n - 1] = 0.0;
    }
  }
}

// ------------------------------------------------------- tridiagonal eigenvalues
// One thread per eigenvalue (csrc/sturm.cuh: FP32 bracket, FP64 Newton for
// isolated eigenvalues, FP64 bisection for clusters).  The Gershgorin bounds
// are reduced over the CTA first.
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
  const skn_sturm::Bounds B = skn_sturm::make_bounds(lo, hi, emax, n);
  __syncthreads();
  for (int j = tid; j < n; j += NT) out[j] = skn_sturm::eigenvalue(V.d, V.e2, V.d32, V.e232, n, j, B);
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

// R = true: real arithmetic on the real parts of H and S (problems whose
// imaginary parts are all zero; the caller routes them).  R = false: complex.
template <bool R>
__global__ void __launch_bounds__(NT, SKN_EIG_MINB) k_eigh_gen(int n_prob, const int32_t* __restrict__ nvec,
                                                 const int64_t* __restrict__ hs_off,
                                                 const int64_t* __restrict__ eig_off,
                                                 const int32_t* __restrict__ order, double2* H, double2* S,
                                                 double* __restrict__ eig, int32_t* __restrict__ status,
                                                 int32_t* __restrict__ counter, int max_n, int use_smem_mats,
                                                 double* __restrict__ tri_all, int64_t n_rows) {
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
    V.v = reinterpret_cast<double2*>(p); p += 2 * max_n;
    V.d32 = reinterpret_cast<float*>(V.rdiag);
    V.e232 = V.d32 + max_n;
  }
  double2* Hs = reinterpret_cast<double2*>(smem + 16 + 4 * NW + 2 * NT + 3 * max_n + (max_n & 1) + 4 * max_n);
  double2* Ss = Hs + SMEM_LDA * SMEM_N;
  double2* tileA = Hs + SMEM_REGION;      // second panel tile of the blocked factorisations
  __shared__ int s_idx;
  for (;;) {
    if (tid == 0) s_idx = atomicAdd(counter, 1);
    __syncthreads();
    const int idx = s_idx;
    __syncthreads();
    if (idx >= n_prob) break;
    const int p = order[idx];
    const int n = nvec[p];
    // A problem larger than the launch's max_n would overrun the shared-memory vectors, and one whose
    // eigenvalue rows end past n_rows would overrun the tridiagonal rows: refuse it, touch nothing.
    if (n < 0 || n > max_n || eig_off[p] < 0 || eig_off[p] + n > n_rows) {
      if (tid == 0) status[p] = SKN_ERR_CAPACITY;
      __syncthreads();
      continue;
    }
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
    // problems staged in shared memory (n <= SMEM_N < NB) are one panel: the unblocked steps
    const bool blocked = SKN_EIG_BLOCKED && !in_smem && n > NB;
    const bool ok = blocked ? cholesky_blocked<R>(Sa, lda, n, V, Hs) : cholesky_lower<R>(Sa, lda, n, V);
    if (!ok) {
      for (int j = tid; j < n; j += NT) eig[eig_off[p] + j] = __longlong_as_double(0x7ff8000000000000LL);
      if (tid == 0) status[p] = SKN_ERR_NOT_SPD;
      __syncthreads();
      continue;
    }
    double* tri = tri_all != nullptr ? tri_all + 4 * eig_off[p] : nullptr;
    if (blocked)
      hegst_blocked<R>(Ha, lda, Sa, lda, n, V, Hs, tileA);
    else
      hegs2_lower<R>(Ha, lda, Sa, lda, n, V, in_smem ? nullptr : Hs);
    hetd2_lower<R>(Ha, lda, n, V, tri);
    if (n == 1 && tid == 0) V.d[0] = Ha[0].x;
    __syncthreads();
    tridiag_eigenvalues(n, V, eig + eig_off[p]);
    if (tri != nullptr && in_smem) {   // reflectors and L must outlive the shared-memory stage
      for (int e = tid; e < n * n; e += NT) {
        const int i = e % n, j = e / n;
        if (i >= j) {
          Hg[e] = Ha[i + j * lda];
          Sg[e] = Sa[i + j * lda];
        }
      }
    }
    if (tid == 0) status[p] = SKN_OK;
    __syncthreads();
  }
}


// ============================================================= eigenvectors
// Eigenvectors of H x = e S x for problems whose values kernel kept the
// reflectors (lower triangle of H), tau, the tridiagonal (d, e) and L (in S):
//   1. inverse iteration on T - e_j I (Gaussian elimination with partial
//      pivoting on the tridiagonal, two solves from a pseudo-random start),
//      one thread per eigenvalue; vectors of eigenvalues closer than 1e-9 of
//      the spectrum's scale are re-orthogonalised (modified Gram-Schmidt, twice);
//   2. y = Q z with Q = H_0 H_1 ... H_{n-2} (reflectors applied last first);
//   3. x = L^-H y, so x^H S x = 1.
// Vectors are written row-major per problem: vec[i*n + j] is component i of
// eigenvector j (the reference's eigh column convention).
constexpr int VNT = 128;
constexpr int VNW = VNT / 32;

__device__ __forceinline__ double hash_unit(unsigned a, unsigned b) {
  unsigned h = a * 0x9E3779B1u ^ (b + 0x7F4A7C15u) * 0x85EBCA77u;
  h ^= h >> 15; h *= 0x2C1B3C6Du; h ^= h >> 12; h *= 0x297A2D39u; h ^= h >> 15;
  return (double)((int)(h & 0xFFFFFF) - 0x800000) * (1.0 / 8388608.0);   // [-1, 1)
}

__device__ double vblock_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int i = 0; i < VNW; ++i) t += red[i];
  return t;
}

__global__ void __launch_bounds__(VNT) k_eigvec(int n_prob, const int32_t* __restrict__ nvec,
                                                const int64_t* __restrict__ hs_off, const int64_t* __restrict__ eig_off,
                                                const int32_t* __restrict__ order, const double2* __restrict__ H,
                                                const double2* __restrict__ S, const double* __restrict__ eig,
                                                const double* __restrict__ tri_all, const int32_t* __restrict__ status,
                                                double2* __restrict__ vec, double* __restrict__ scratch,
                                                int32_t* __restrict__ counter, int max_n) {
  extern __shared__ double smem[];
  double* red = smem;                                      // 2*VNW
  double* d = smem + 2 * VNW;                              // max_n
  double* e = d + max_n;                                   // max_n
  double2* col = reinterpret_cast<double2*>(e + max_n);  // max_n (offset 2*VNW + 2*max_n doubles: even)
  __shared__ int s_idx;
  const int tid = threadIdx.x;
  const int64_t sstride = (int64_t)max_n * VNT;
  double* su = scratch + (int64_t)blockIdx.x * 5 * sstride;   // rows i: [i*VNT + tid]
  double* s_ru1 = su;                 // 1 / u1
  double* s_u2 = su + sstride;
  double* s_u3 = su + 2 * sstride;
  double* s_m = su + 3 * sstride;
  double* s_pv = su + 4 * sstride;    // 1.0 where rows were swapped
  for (;;) {
    if (tid == 0) s_idx = atomicAdd(counter, 1);
    __syncthreads();
    const int idx = s_idx;
    __syncthreads();
    if (idx >= n_prob) break;
    const int p = order[idx];
    const int n = nvec[p];
    double2* Y = vec + hs_off[p];
    if (status[p] != SKN_OK) {
      // a problem the values kernel refused for its size keeps its buffers untouched
      if (status[p] != SKN_ERR_CAPACITY)
        for (int q = tid; q < n * n; q += VNT) Y[q] = make_double2(__longlong_as_double(0x7ff8000000000000LL), 0.0);
      __syncthreads();
      continue;
    }
    const double* tri = tri_all + 4 * eig_off[p];
    const double* w = eig + eig_off[p];
    const double2* A = H + hs_off[p];
    const double2* L = S + hs_off[p];
    for (int i = tid; i < n; i += VNT) {
      d[i] = tri[i];
      e[i] = tri[n + i];
    }
    __syncthreads();
    double scale = 0.0;
    for (int i = tid; i < n; i += VNT) scale = fmax(scale, fabs(w[i]));
    for (int o = 16; o > 0; o >>= 1) scale = fmax(scale, __shfl_xor_sync(0xffffffffu, scale, o));
    __syncthreads();
    if ((tid & 31) == 0) red[tid >> 5] = scale;
    __syncthreads();
    scale = red[0];
    for (int q = 1; q < VNW; ++q) scale = fmax(scale, red[q]);
    scale = fmax(scale, 1e-300);
    const double pivmin = 1e-300 * fmax(1.0, scale);

    // ---- 1. inverse iteration, one eigenvalue per thread
    for (int j0 = 0; j0 < n; j0 += VNT) {
      const int j = j0 + tid;
      if (j < n) {
        const double lam = w[j];
        double u1 = d[0] - lam, u2 = (n > 1) ? e[0] : 0.0;
        double rmax = 0.0;                 // largest |1 / pivot|
        for (int i = 0; i < n - 1; ++i) {
          const double c = e[i];
          const double a1 = d[i + 1] - lam;
          const double b1 = (i + 1 < n - 1) ? e[i + 1] : 0.0;
          double m, r1, r2, r3, pv;
          if (fabs(u1) >= fabs(c)) {
            if (fabs(u1) < pivmin) u1 = (u1 < 0.0) ? -pivmin : pivmin;
            m = c / u1;
            r1 = u1; r2 = u2; r3 = 0.0; pv = 0.0;
            u1 = a1 - m * u2;
            u2 = b1;
          } else {
            m = u1 / c;
            r1 = c; r2 = a1; r3 = b1; pv = 1.0;
            u1 = u2 - m * a1;
            u2 = -m * b1;
          }
          s_ru1[i * VNT + tid] = 1.0 / r1;
          rmax = fmax(rmax, fabs(1.0 / r1));
          s_u2[i * VNT + tid] = r2;
          s_u3[i * VNT + tid] = r3;
          s_m[i * VNT + tid] = m;
          s_pv[i * VNT + tid] = pv;
        }
        if (fabs(u1) < pivmin) u1 = (u1 < 0.0) ? -pivmin : pivmin;
        s_ru1[(n - 1) * VNT + tid] = 1.0 / u1;
        rmax = fmax(rmax, fabs(1.0 / u1));
        // A lam exact to the last bit (the Newton step can land on the eigenvalue) leaves a pivot at the
        // 1e-300 floor, and a solve then grows the vector by up to 1 / pivot: its sum of squares overflowed
        // and the eigenvector came out NaN.  Every solve's right-hand side is therefore scaled by
        // ysc = 2^-e with 2^e >= rmax, which keeps the solution near unit size; a power of two scales
        // exactly, so without a tiny pivot the normalised vectors are bitwise what they were unscaled.
        int rex = 0;
        frexp(rmax, &rex);
        const double ysc = rex > 0 ? ldexp(1.0, -rex) : 1.0;
        // y lives in the real parts of column j of Y
        for (int i = 0; i < n; ++i) Y[(int64_t)i * n + j] = make_double2(hash_unit(j, i) * ysc, 0.0);
        for (int it = 0; it < 2; ++it) {
          for (int i = 0; i < n - 1; ++i) {
            const double m = s_m[i * VNT + tid];
            const double yi = Y[(int64_t)i * n + j].x, yn = Y[(int64_t)(i + 1) * n + j].x;
            if (s_pv[i * VNT + tid] != 0.0) {
              Y[(int64_t)i * n + j].x = yn;
              Y[(int64_t)(i + 1) * n + j].x = yi - m * yn;
            } else {
              Y[(int64_t)(i + 1) * n + j].x = yn - m * yi;
            }
          }
          double x2 = 0.0, x1 = 0.0, nrm = 0.0;
          for (int i = n - 1; i >= 0; --i) {
            const double xi = (Y[(int64_t)i * n + j].x - s_u2[i * VNT + tid] * x1 - s_u3[i * VNT + tid] * x2) *
                              s_ru1[i * VNT + tid];
            Y[(int64_t)i * n + j].x = xi;
            nrm = fma(xi, xi, nrm);
            x2 = x1;
            x1 = xi;
          }
          if (!(nrm > 0.0 && nrm <= 1.7976931348623157e308)) {   // vanished, overflowed or NaN: restart from e_j
            for (int i = 0; i < n; ++i) Y[(int64_t)i * n + j].x = (i == j) ? ysc : 0.0;
            nrm = ysc * ysc;
          }
          // normalised, and scaled by ysc again when it is the next solve's right-hand side
          const double inv = (it == 0 ? ysc : 1.0) / sqrt(nrm);
          for (int i = 0; i < n; ++i) Y[(int64_t)i * n + j].x *= inv;
        }
      }
    }
    __syncthreads();
    // ---- clusters: modified Gram-Schmidt (twice) within runs of close eigenvalues
    {
      const double ctol = 1e-9 * scale;
      int j = 1;
      while (j < n) {
        if (w[j] - w[j - 1] > ctol) { ++j; continue; }
        int j0 = j - 1, j1 = j + 1;
        while (j1 < n && w[j1] - w[j1 - 1] <= ctol) ++j1;
        for (int pass = 0; pass < 2; ++pass) {
          for (int q = j0; q < j1; ++q) {
            for (int r = j0; r < q; ++r) {
              double dp = 0.0;
              for (int i = tid; i < n; i += VNT) dp = fma(Y[(int64_t)i * n + r].x, Y[(int64_t)i * n + q].x, dp);
              dp = vblock_sum(dp, red);
              for (int i = tid; i < n; i += VNT) Y[(int64_t)i * n + q].x -= dp * Y[(int64_t)i * n + r].x;
              __syncthreads();
            }
            double nn = 0.0;
            for (int i = tid; i < n; i += VNT) nn = fma(Y[(int64_t)i * n + q].x, Y[(int64_t)i * n + q].x, nn);
            nn = vblock_sum(nn, red);
            const double inv = 1.0 / sqrt(nn);
            for (int i = tid; i < n; i += VNT) Y[(int64_t)i * n + q].x *= inv;
            __syncthreads();
          }
        }
        j = j1;
      }
    }
    __syncthreads();
    // ---- 2. back-transformation y = Q z
    for (int k = n - 2; k >= 0; --k) {
      const double2 tau = make_double2(tri[2 * n + 2 * k], tri[2 * n + 2 * k + 1]);
      if (tau.x == 0.0 && tau.y == 0.0) continue;
      const int m = n - k - 1;
      for (int r = tid; r < m; r += VNT)
        col[r] = (r == 0) ? make_double2(1.0, 0.0) : A[(k + 1 + r) + (int64_t)k * n];
      __syncthreads();
      for (int jj = tid; jj < n; jj += VNT) {
        double2 s0 = make_double2(0.0, 0.0), s1 = s0, s2 = s0, s3 = s0;
        int r = 0;
        for (; r + 3 < m; r += 4) {
          const double2 y0 = Y[(int64_t)(k + 1 + r) * n + jj], y1 = Y[(int64_t)(k + 2 + r) * n + jj];
          const double2 y2 = Y[(int64_t)(k + 3 + r) * n + jj], y3 = Y[(int64_t)(k + 4 + r) * n + jj];
          s0 = cfma_conj(col[r], y0, s0);
          s1 = cfma_conj(col[r + 1], y1, s1);
          s2 = cfma_conj(col[r + 2], y2, s2);
          s3 = cfma_conj(col[r + 3], y3, s3);
        }
        for (; r < m; ++r) s0 = cfma_conj(col[r], Y[(int64_t)(k + 1 + r) * n + jj], s0);
        s0.x += s1.x + (s2.x + s3.x);
        s0.y += s1.y + (s2.y + s3.y);
        const double2 ts = cmul(tau, s0);          // y -= tau v (v^H y)
        for (int q = 0; q < m; ++q) {
          double2 y = Y[(int64_t)(k + 1 + q) * n + jj];
          y = cfms_conj(col[q], make_double2(ts.x, -ts.y), y);
          Y[(int64_t)(k + 1 + q) * n + jj] = y;
        }
      }
      __syncthreads();
    }
    // ---- 3. x = L^-H y (backward substitution, one column per thread)
    for (int i = n - 1; i >= 0; --i) {
      const int m = n - i - 1;
      for (int r = tid; r < m; r += VNT) col[r] = L[(i + 1 + r) + (int64_t)i * n];
      if (tid == 0) col[max_n - 1] = L[i + (int64_t)i * n];
      __syncthreads();
      const double rl = 1.0 / col[max_n - 1].x;
      for (int jj = tid; jj < n; jj += VNT) {
        double2 acc0 = Y[(int64_t)i * n + jj], acc1 = make_double2(0.0, 0.0), acc2 = acc1, acc3 = acc1;
        int r = 0;
        for (; r + 3 < m; r += 4) {
          const double2 y0 = Y[(int64_t)(i + 1 + r) * n + jj], y1 = Y[(int64_t)(i + 2 + r) * n + jj];
          const double2 y2 = Y[(int64_t)(i + 3 + r) * n + jj], y3 = Y[(int64_t)(i + 4 + r) * n + jj];
          acc0 = cfms_conj_l(col[r], y0, acc0);
          acc1 = cfms_conj_l(col[r + 1], y1, acc1);
          acc2 = cfms_conj_l(col[r + 2], y2, acc2);
          acc3 = cfms_conj_l(col[r + 3], y3, acc3);
        }
        for (; r < m; ++r) acc0 = cfms_conj_l(col[r], Y[(int64_t)(i + 1 + r) * n + jj], acc0);
        Y[(int64_t)i * n + jj] = make_double2((acc0.x + acc1.x + (acc2.x + acc3.x)) * rl,
                                              (acc0.y + acc1.y + (acc2.y + acc3.y)) * rl);
      }
      __syncthreads();
    }
  }
}
}  // namespace
}  // namespace SKN_EIG_NS
using namespace SKN_EIG_NS;

// Dynamic shared-memory limits are per-function attributes.  They are set to
// the largest size any call can request (max_n = MAX_N), so concurrent calls
// from several host threads never lower the limit under another's launch.
static size_t eig_smem_bytes(int mn) {
  return sizeof(double) * (16 + 4 * NW + 2 * NT + 3 * (size_t)mn + (mn & 1) + 4 * (size_t)mn) +
         (SMEM_REGION + (SKN_EIG_BLOCKED ? NB * LDT : 0)) * sizeof(double2);
}
static size_t vec_smem_bytes(int mn) {
  return sizeof(double) * (2 * VNW + 2 * (size_t)mn + 2) + sizeof(double2) * (size_t)mn;
}
static cudaError_t set_smem_limit_once() {
  cudaError_t e = cudaFuncSetAttribute(k_eigh_gen<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)eig_smem_bytes(MAX_N));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_eigh_gen<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)eig_smem_bytes(MAX_N));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_eigvec, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)vec_smem_bytes(MAX_N));
}

// Values-only launch of k_eigh_gen<R> over a persistent grid (all problems of the call).
template <bool R>
static int launch_values(int n_prob, const int32_t* n, const int64_t* hs_off, const int64_t* eig_off,
                         const int32_t* order, double* H, double* S, double* eig, int32_t* status,
                         int32_t* work_counter, int max_n, cudaStream_t stream) {
  if (n_prob < 0 || max_n < 0) return SKN_ERR_ARG;
  if (n_prob == 0) return SKN_OK;
  if (!n || !hs_off || !eig_off || !order || !H || !S || !eig || !status || !work_counter) return SKN_ERR_ARG;
  if (max_n > MAX_N) return SKN_ERR_CAPACITY;
  const int mn = max_n < 1 ? 1 : max_n;
  const size_t smem = eig_smem_bytes(mn);
  if (set_smem_limit_once() != cudaSuccess) return SKN_ERR_CUDA;
  int per_sm = 0, dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_eigh_gen<R>, NT, smem) != cudaSuccess || per_sm < 1)
    return SKN_ERR_CUDA;
  int grid = sms * per_sm;
  if (grid > n_prob) grid = n_prob;
  if (cudaMemsetAsync(work_counter, 0, sizeof(int32_t), stream) != cudaSuccess) return SKN_ERR_CUDA;
  k_eigh_gen<R><<<grid, NT, smem, stream>>>(n_prob, n, hs_off, eig_off, order, (double2*)H, (double2*)S, eig,
                                            status, work_counter, mn, 1, nullptr, INT64_MAX);
  return cudaPeekAtLastError() == cudaSuccess ? SKN_OK : SKN_ERR_CUDA;
}

// A translation unit that includes this file for its kernels alone defines
// SKN_EIG_KERNELS_ONLY and provides its own entry points.
#ifndef SKN_EIG_KERNELS_ONLY
extern "C" int SKN_EXPORT(skn_eigh_gen_batched)(int n_prob, const int32_t* n, const int64_t* hs_off, const int64_t* eig_off,
                                    const int32_t* order, double* H, double* S, double* eig, int32_t* status,
                                    int32_t* work_counter, int max_n, cudaStream_t stream) {
  return launch_values<false>(n_prob, n, hs_off, eig_off, order, H, S, eig, status, work_counter, max_n, stream);
}

extern "C" int SKN_EXPORT(skn_eigh_gen_batched_real)(int n_prob, const int32_t* n, const int64_t* hs_off,
                                                    const int64_t* eig_off, const int32_t* order, double* H,
                                                    double* S, double* eig, int32_t* status,
                                                    int32_t* work_counter, int max_n, cudaStream_t stream) {
  return launch_values<true>(n_prob, n, hs_off, eig_off, order, H, S, eig, status, work_counter, max_n, stream);
}

// CTAs of the vector stage: as many as fit on the GPU at once (the stage is latency-bound, so
// occupancy matters), but no more than the problems, and no more than keep the inverse-iteration
// scratch (5 * max_n * VNT doubles per CTA) within VEC_SCRATCH_BUDGET.  Each problem is solved by
// one CTA, so the results do not depend on the grid.
constexpr int64_t VEC_SCRATCH_BUDGET = (int64_t)2 << 30;
static int vec_grid(int n_prob, int max_n) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms < 1) sms = 1;
  const int mn = max_n < 1 ? 1 : max_n;
  if (set_smem_limit_once() != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_eigvec, VNT, vec_smem_bytes(mn)) != cudaSuccess ||
      per_sm < 1)
    per_sm = 2;
  int64_t g = (int64_t)sms * per_sm;
  const int64_t per_cta = (int64_t)5 * mn * VNT * (int64_t)sizeof(double);
  const int64_t cap = VEC_SCRATCH_BUDGET / per_cta;
  if (g > cap) g = cap;
  if (g < sms) g = sms < n_prob ? sms : n_prob;      // never fewer than one CTA per SM (or per problem)
  if (g > n_prob) g = n_prob;
  return g > 0 ? (int)g : 1;
}

extern "C" int SKN_EXPORT(skn_eigh_vectors_scratch_bytes)(int n_prob, int max_n, int64_t* bytes) {
  if (!bytes || max_n < 0 || n_prob < 0) return SKN_ERR_ARG;
  *bytes = (int64_t)vec_grid(n_prob, max_n) * 5 * (int64_t)(max_n < 1 ? 1 : max_n) * VNT * (int64_t)sizeof(double);
  return SKN_OK;
}

extern "C" int SKN_EXPORT(skn_eigh_gen_vectors)(int n_prob, const int32_t* n, const int64_t* hs_off, const int64_t* eig_off,
                                    const int32_t* order, double* H, double* S, double* eig, double* vec,
                                    int32_t* status, double* tri, double* scratch, int64_t scratch_bytes,
                                    int32_t* work_counter, int max_n, cudaStream_t stream) {
  if (n_prob < 0 || max_n < 0) return SKN_ERR_ARG;
  if (n_prob == 0) return SKN_OK;
  if (!n || !hs_off || !eig_off || !order || !H || !S || !eig || !vec || !status || !tri || !scratch ||
      !work_counter)
    return SKN_ERR_ARG;
  if (max_n > MAX_N) return SKN_ERR_CAPACITY;
  int64_t need = 0;
  SKN_EXPORT(skn_eigh_vectors_scratch_bytes)(n_prob, max_n, &need);
  if (scratch_bytes < need) return SKN_ERR_CAPACITY;
  const int mn = max_n < 1 ? 1 : max_n;
  const int use_smem_mats = 1;
  const size_t smem = eig_smem_bytes(mn);
  if (set_smem_limit_once() != cudaSuccess) return SKN_ERR_CUDA;
  int per_sm = 0, dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_eigh_gen<false>, NT, smem) != cudaSuccess ||
      per_sm < 1)
    return SKN_ERR_CUDA;
  int grid = sms * per_sm;
  if (grid > n_prob) grid = n_prob;
  if (cudaMemsetAsync(work_counter, 0, 2 * sizeof(int32_t), stream) != cudaSuccess) return SKN_ERR_CUDA;
  k_eigh_gen<false><<<grid, NT, smem, stream>>>(n_prob, n, hs_off, eig_off, order, (double2*)H, (double2*)S, eig, status,
                                         work_counter, mn, use_smem_mats, tri, INT64_MAX);
  if (cudaPeekAtLastError() != cudaSuccess) return SKN_ERR_CUDA;
  const size_t vsmem = sizeof(double) * (2 * VNW + 2 * (size_t)mn + 2) + sizeof(double2) * (size_t)mn;

  k_eigvec<<<vec_grid(n_prob, mn), VNT, vsmem, stream>>>(n_prob, n, hs_off, eig_off, order, (const double2*)H,
                                                     (const double2*)S, eig, tri, status, (double2*)vec, scratch,
                                                     work_counter + 1, mn);
  return cudaPeekAtLastError() == cudaSuccess ? SKN_OK : SKN_ERR_CUDA;
}
#endif  // SKN_EIG_KERNELS_ONLY
