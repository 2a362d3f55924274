// Generalized Hermitian eigenvalues of large problems: one thread-block
// cluster per problem.
//
// Same steps as k_eigh_gen in eigh.cu (unit diagonal for zero rows, Cholesky
// S = L L^H, reduction to L^-1 H L^-H in zhegs2 column order, zhetd2
// Householder tridiagonalisation, Sturm-count eigenvalues), but the C CTAs of a
// cluster, one per SM, share one problem held in global memory: every
// O(m^2)-per-column loop is split over all C*CNT threads of the cluster,
// phases are separated by cluster barriers, and reductions go through
// distributed shared memory in a fixed rank order, so every CTA derives
// bitwise the same Householder scalars.  The hardware co-schedules the CTAs of
// a cluster, so a barrier never waits on a CTA that is not running.  Data
// written by another CTA is read through L2 (ld.global.cg).
//
// Cost: 32/3 n^3 FP64 flops per problem.  One SM delivers ~8 GFLOP/s FP64,
// so a single CTA needs ~1.3 s at n = 1000 and ~20 min at n = 9000; a
// 16-CTA cluster divides that by up to 16.  Per column the cluster pays
// about 9 + m/64 barriers (the triangular solve of the reduction advances
// 64 rows per barrier: each CTA stages the 64x64 diagonal block of L in shared
// memory and solves it itself).
#include "skn_common.cuh"
#include "sturm.cuh"
#include <cooperative_groups.h>

namespace cg = cooperative_groups;

#ifndef SKN_CL_NT
#define SKN_CL_NT 512
#endif

namespace {

constexpr int CNT = SKN_CL_NT;           // threads per CTA
constexpr int CNW = CNT / 32;
constexpr int CH = 64;                   // rows of the triangular solve per cluster barrier
constexpr int LBLD = CH + 1;             // leading dimension of the staged diagonal block of L
constexpr int MAX_CLUSTER = 16;
constexpr int VEC_DOUBLES = 9;           // per-orbital doubles of cluster scratch (see CV)
// Doubles of scratch per cluster, a multiple of 32 (256 bytes) so every
// cluster's complex vectors stay 16-byte aligned whatever max_n is.
__host__ __device__ __forceinline__ int64_t cluster_stride(int max_n) {
  return ((int64_t)VEC_DOUBLES * max_n + 31) / 32 * 32;
}
constexpr int LARGE_MAX_N = 9216;        // d, e^2 and their FP32 copies (24 bytes per row) in shared memory
constexpr int SMEM_FLOOR = 116 * 1024;   // at least half an SM's shared memory: one CTA per SM
static_assert(CH * LBLD * 16 + CH * 8 <= SMEM_FLOOR, "staged block of L exceeds the shared-memory floor");
static_assert(CNT * 16 <= SMEM_FLOOR, "partial sums exceed the shared-memory floor");

struct CV {   // per-cluster vectors in global memory
  double2* v;     // working column / Householder vector
  double2* w;     // L column / hemv result
  double2* x;     // right-hand side of the triangular solve
  double* d;      // tridiagonal diagonal
  double* e2;     // squared off-diagonal
  double* rdiag;  // 1 / L_kk
};

__device__ __forceinline__ double2 ldc(const double2* p) { return __ldcg(p); }
__device__ __forceinline__ double ldc(const double* p) { return __ldcg(p); }

// Cluster-wide sum of two doubles per thread, same value in every CTA.  Slots
// alternate between two buffers, so one cluster barrier per reduction suffices:
// a slot is rewritten two reductions later, after every CTA has passed the
// barrier of the reduction in between.
struct ClusterSum {
  double* slots;   // shared [4]
  double* warp;    // shared [2 * CNW]
  int parity;
  __device__ void sum2(cg::cluster_group& cl, double& a, double& b) {
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) {
      warp[threadIdx.x >> 5] = a;
      warp[CNW + (threadIdx.x >> 5)] = b;
    }
    __syncthreads();
    double* slot = slots + 2 * parity;
    if (threadIdx.x == 0) {
      double sa = 0.0, sb = 0.0;
      for (int i = 0; i < CNW; ++i) {
        sa += warp[i];
        sb += warp[CNW + i];
      }
      slot[0] = sa;
      slot[1] = sb;
    }
    cl.sync();
    double ta = 0.0, tb = 0.0;
    const unsigned C = cl.num_blocks();
    for (unsigned r = 0; r < C; ++r) {
      const double* rs = cl.map_shared_rank(slot, r);
      ta += rs[0];
      tb += rs[1];
    }
    a = ta;
    b = tb;
    parity ^= 1;
  }
};

// Packed lower-triangle updates of the m x m block at T, entries split over
// the cluster's threads, four loads in flight per thread.
//   MODE 0: T -= x x^H           (Cholesky trailing update)
//   MODE 1: T -= x y^H + y x^H   (rank-2 update)
template <int MODE>
__device__ void tri_update(double2* T, int lda, int m, const double2* x, const double2* y, int gt, int GT) {
  constexpr int U = 4;
  const int tri = m * (m + 1) / 2;
  for (int e0 = gt; e0 < tri; e0 += GT * U) {
    int off[U], ii[U], jj[U];
    double2 a[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int e = e0 + u * GT;
      if (e < tri) {
        tri_index(e, m, ii[u], jj[u]);
        off[u] = ii[u] + jj[u] * lda;
        a[u] = ldc(T + off[u]);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (e0 + u * GT < tri) {
        if (MODE == 0) {
          T[off[u]] = cfms_conj(ldc(x + ii[u]), ldc(x + jj[u]), a[u]);
        } else {
          const double2 v = cfms_conj(ldc(x + ii[u]), ldc(y + jj[u]), a[u]);
          T[off[u]] = cfms_conj(ldc(y + ii[u]), ldc(x + jj[u]), v);
        }
      }
    }
  }
}

__device__ __forceinline__ double2 csub_mul(double2 v, double2 x, double2 l) {   // v - x * l
  v.x = fma(-x.x, l.x, v.x);
  v.x = fma(x.y, l.y, v.x);
  v.y = fma(-x.x, l.y, v.y);
  v.y = fma(-x.y, l.x, v.y);
  return v;
}

__global__ void __launch_bounds__(CNT, 1) k_eigh_cluster(int n_prob, const int32_t* __restrict__ nvec,
                                                         const int64_t* __restrict__ hs_off,
                                                         const int64_t* __restrict__ eig_off,
                                                         const int32_t* __restrict__ order, double2* H, double2* S,
                                                         double* __restrict__ eig, int32_t* __restrict__ status,
                                                         int32_t* __restrict__ counter, double* scratch, int max_n) {
  cg::cluster_group cl = cg::this_cluster();
  __shared__ double red_slots[4];
  __shared__ double red_warp[3 * CNW];
  __shared__ double2 xs[CH];
  __shared__ double sc[4];
  __shared__ int s_idx;
  const int tid = threadIdx.x;
  const int rank = (int)cl.block_rank();
  const int C = (int)cl.num_blocks();
  const int gt = rank * CNT + tid, GT = C * CNT;
  const int cid = blockIdx.x / C;
  const bool lead = rank == 0 && tid == 0;
  ClusterSum R{red_slots, red_warp, 0};
  CV V;
  {
    double* base = scratch + (int64_t)cid * cluster_stride(max_n);
    V.v = reinterpret_cast<double2*>(base);
    V.w = V.v + max_n;
    V.x = V.w + max_n;
    V.d = base + 6 * (int64_t)max_n;
    V.e2 = V.d + max_n;
    V.rdiag = V.e2 + max_n;
  }
  extern __shared__ double dyn[];
  // Dynamic shared memory, reused by phase: the staged diagonal block of L and
  // 1/diag (reduction), partial sums of the Hermitian product (tridiagonalisation),
  // the copies of the tridiagonal: 24 bytes per row (bisection).
  double2* Lb = reinterpret_cast<double2*>(dyn);          // CH x LBLD
  double* rds = reinterpret_cast<double*>(Lb + CH * LBLD);   // CH
  double2* hpart = reinterpret_cast<double2*>(dyn);       // CNT
  double* sd = dyn;
  double* se2 = sd + max_n;
  float* sd32 = reinterpret_cast<float*>(se2 + max_n);
  float* se232 = sd32 + max_n;
  for (;;) {
    if (lead) s_idx = atomicAdd(counter, 1);
    cl.sync();
    const int idx = *cl.map_shared_rank(&s_idx, 0);
    cl.sync();   // rank 0 rewrites s_idx only after every CTA has read it
    if (idx >= n_prob) break;
    const int p = order[idx];
    const int n = nvec[p];
    double2* A = H + hs_off[p];
    double2* B = S + hs_off[p];
    const int lda = n;

    // unit diagonal for rows that are entirely zero (eighb's aux option)
    for (int i = gt; i < n; i += GT) {
      for (int which = 0; which < 2; ++which) {
        double2* M = which ? B : A;
        bool zero = true;
        for (int j = 0; j < n && zero; ++j) {
          const double2 v = (j <= i) ? ldc(M + i + (int64_t)j * lda) : ldc(M + j + (int64_t)i * lda);
          zero = is_zero_bits(v.x) && is_zero_bits(v.y);
        }
        if (zero) M[i + (int64_t)i * lda].x += 1.0;
      }
    }
    cl.sync();

    // ------------------------------------------------------------ Cholesky of S
    bool ok = true;
    for (int k = 0; k < n; ++k) {
      if (tid == 0) {
        const double a = ldc(B + k + (int64_t)k * lda).x;
        const bool good = (a > 0.0) && is_finite_bits(a);
        const double dk = good ? sqrt(a) : 1.0;
        sc[0] = dk;
        sc[1] = 1.0 / dk;
        sc[2] = good ? 1.0 : 0.0;
      }
      __syncthreads();
      if (sc[2] == 0.0) {   // every CTA read the same diagonal entry
        ok = false;
        break;
      }
      const double rd = sc[1];
      const int m = n - k - 1;
      double2* col = B + (k + 1) + (int64_t)k * lda;
      for (int i = gt; i < m; i += GT) {
        const double2 v = cscale(ldc(col + i), rd);
        col[i] = v;
        V.v[i] = v;
      }
      cl.sync();
      if (lead) {
        B[k + (int64_t)k * lda] = make_double2(sc[0], 0.0);
        V.rdiag[k] = rd;
      }
      tri_update<0>(B + (k + 1) + (int64_t)(k + 1) * lda, lda, m, V.v, nullptr, gt, GT);
      cl.sync();
    }
    if (!ok) {
      for (int j = gt; j < n; j += GT) eig[eig_off[p] + j] = __longlong_as_double(0x7ff8000000000000LL);
      if (lead) status[p] = SKN_ERR_NOT_SPD;
      cl.sync();
      continue;
    }

    // ---------------------------------------- reduction C = L^-1 H L^-H (zhegs2 order)
    for (int k = 0; k < n; ++k) {
      const double rd = ldc(V.rdiag + k);
      const double akk = ldc(A + k + (int64_t)k * lda).x * (rd * rd);
      const double ct = -0.5 * akk;
      const int m = n - k - 1;
      if (m == 0) {
        cl.sync();   // every thread has read A[k][k]
        if (lead) A[k + (int64_t)k * lda] = make_double2(akk, 0.0);
        break;
      }
      double2* acol = A + (k + 1) + (int64_t)k * lda;
      const double2* bcol = B + (k + 1) + (int64_t)k * lda;
      for (int i = gt; i < m; i += GT) {
        const double2 bi = ldc(bcol + i);
        double2 v = cscale(ldc(acol + i), rd);
        v.x = fma(ct, bi.x, v.x);
        v.y = fma(ct, bi.y, v.y);
        V.v[i] = v;
        V.w[i] = bi;
      }
      cl.sync();
      if (lead) A[k + (int64_t)k * lda] = make_double2(akk, 0.0);
      tri_update<1>(A + (k + 1) + (int64_t)(k + 1) * lda, lda, m, V.v, V.w, gt, GT);
      for (int i = gt; i < m; i += GT) {   // second axpy into x (v and w stay intact for the update above)
        double2 v = ldc(V.v + i);
        const double2 bi = ldc(V.w + i);
        v.x = fma(ct, bi.x, v.x);
        v.y = fma(ct, bi.y, v.y);
        V.x[i] = v;
      }
      cl.sync();
      // x <- L22^-1 x.  Every CTA stages the CH x CH diagonal block of L22 and
      // 1/diag in shared memory and solves the chunk itself (warp 0 per 32 rows,
      // the CTA updating the chunk's later rows), then the cluster applies the
      // solved chunk to the rows below it.
      const double2* L = B + (k + 1) + (int64_t)(k + 1) * lda;
      const double* rdl = V.rdiag + k + 1;
      for (int c0 = 0; c0 < m; c0 += CH) {
        const int cm = min(CH, m - c0);
        for (int e = tid; e < CH * CH; e += CNT) {
          const int r = e % CH, c = e / CH;
          if (r < cm && c <= r) Lb[r + c * LBLD] = ldc(L + (c0 + r) + (int64_t)(c0 + c) * lda);
        }
        for (int i = tid; i < cm; i += CNT) {
          xs[i] = ldc(V.x + c0 + i);
          rds[i] = ldc(rdl + c0 + i);
        }
        __syncthreads();
        for (int s0 = 0; s0 < cm; s0 += 32) {
          const int sm = min(32, cm - s0);
          if (tid < 32) {
            const int lane = tid;
            double2 xv = (lane < sm) ? xs[s0 + lane] : make_double2(0.0, 0.0);
            for (int i = 0; i < sm; ++i) {
              if (lane == i) xv = cscale(xv, rds[s0 + i]);
              double2 xi;
              xi.x = __shfl_sync(0xffffffffu, xv.x, i);
              xi.y = __shfl_sync(0xffffffffu, xv.y, i);
              if (lane > i && lane < sm) xv = csub_mul(xv, xi, Lb[(s0 + lane) + (s0 + i) * LBLD]);
            }
            if (lane < sm) xs[s0 + lane] = xv;
          }
          __syncthreads();
          for (int r = s0 + sm + tid; r < cm; r += CNT) {
            double2 v0 = xs[r], v1 = make_double2(0.0, 0.0);
            int i = 0;
            for (; i + 1 < sm; i += 2) {
              v0 = csub_mul(v0, xs[s0 + i], Lb[r + (s0 + i) * LBLD]);
              v1 = csub_mul(v1, xs[s0 + i + 1], Lb[r + (s0 + i + 1) * LBLD]);
            }
            if (i < sm) v0 = csub_mul(v0, xs[s0 + i], Lb[r + (s0 + i) * LBLD]);
            xs[r] = make_double2(v0.x + v1.x, v0.y + v1.y);
          }
          __syncthreads();
        }
        if (rank == 0)   // nothing else reads or writes column k of A during the solve
          for (int i = tid; i < cm; i += CNT) acol[c0 + i] = xs[i];
        const int rest = m - c0 - cm;
        for (int r = gt; r < rest; r += GT) {
          const int row = c0 + cm + r;
          double2 acc[4] = {ldc(V.x + row), make_double2(0.0, 0.0), make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
          const double2* Lr = L + row + (int64_t)c0 * lda;
          int i = 0;
          for (; i + 7 < cm; i += 8) {
            double2 l[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) l[u] = ldc(Lr + (int64_t)(i + u) * lda);
#pragma unroll
            for (int u = 0; u < 8; ++u) acc[u & 3] = csub_mul(acc[u & 3], xs[i + u], l[u]);
          }
          for (; i < cm; ++i) acc[0] = csub_mul(acc[0], xs[i], ldc(Lr + (int64_t)i * lda));
          V.x[row] = make_double2((acc[0].x + acc[1].x) + (acc[2].x + acc[3].x),
                                  (acc[0].y + acc[1].y) + (acc[2].y + acc[3].y));
        }
        if (rest > 0) cl.sync();
        else __syncthreads();
      }
    }
    cl.sync();

    // ---------------------------------------------------------- tridiagonalisation
    for (int k = 0; k < n - 1; ++k) {
      const int m = n - k - 1;
      double2* x = A + (k + 1) + (int64_t)k * lda;
      double s = 0.0, s_unused = 0.0;
      for (int i = 1 + gt; i < m; i += GT) {
        const double2 xi = ldc(x + i);
        s = fma(xi.x, xi.x, fma(xi.y, xi.y, s));
      }
      R.sum2(cl, s, s_unused);
      const double xnorm2 = s;
      const double2 alpha = ldc(x);
      double beta, taur = 0.0, taui = 0.0, sclr = 0.0, scli = 0.0;
      const bool trivial = (xnorm2 == 0.0 && alpha.y == 0.0);
      if (trivial) {
        beta = alpha.x;
      } else {
        const double nrm = sqrt(fma(alpha.x, alpha.x, fma(alpha.y, alpha.y, xnorm2)));
        beta = alpha.x >= 0.0 ? -nrm : nrm;
        taur = (beta - alpha.x) / beta;
        taui = -alpha.y / beta;
        const double dr = alpha.x - beta, di = alpha.y;
        const double den = 1.0 / fma(dr, dr, di * di);
        sclr = dr * den;
        scli = -di * den;
      }
      if (lead) {
        V.d[k] = ldc(A + k + (int64_t)k * lda).x;
        V.e2[k] = beta * beta;
      }
      if (!trivial) {
        const double2 tau = make_double2(taur, taui);
        const double2 scl = make_double2(sclr, scli);
        for (int i = gt; i < m; i += GT) {
          if (i == 0) {
            V.v[0] = make_double2(1.0, 0.0);
          } else {
            const double2 v = cmul(ldc(x + i), scl);
            V.v[i] = v;
            x[i] = v;
          }
        }
        cl.sync();
        // w = tau * A22 v.  Each CTA owns a contiguous block of rows, 32 rows per
        // warp (lanes on rows, the upper triangle read as the conjugate of the
        // lower); when the block has fewer row groups than the CTA has warps,
        // the warps split the j range and partial sums meet in shared memory.
        const double2* T = A + (k + 1) + (int64_t)(k + 1) * lda;
        double pr = 0.0, pi = 0.0;
        {
          const int per = (m + C - 1) / C;
          const int r0 = min(m, rank * per), r1 = min(m, r0 + per);
          const int G = (r1 - r0 + 31) / 32;
          const int nseg = (G == 0) ? 1 : (G >= CNW ? 1 : CNW / G);
          const int seg = (m + nseg - 1) / nseg;
          const int w = tid >> 5, lane = tid & 31;
          for (int g0 = (nseg == 1 ? w : w % G); g0 < G; g0 += (nseg == 1 ? CNW : G)) {
            const int sg = (nseg == 1) ? 0 : w / G;
            if (sg >= nseg) break;
            const int row = r0 + g0 * 32 + lane;
            const int i = min(row, r1 - 1);
            const int j0 = sg * seg, j1 = min(m, j0 + seg);
            double2 acc[2] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
            int j = j0;
            for (; j + 3 < j1; j += 4) {
              double2 a[4];
#pragma unroll
              for (int u = 0; u < 4; ++u) {
                const int jj = j + u;
                const bool up = jj > i;
                a[u] = up ? ldc(T + jj + (int64_t)i * lda) : ldc(T + i + (int64_t)jj * lda);
                a[u].y = cond_flip(a[u].y, up);
              }
#pragma unroll
              for (int u = 0; u < 4; ++u) acc[u & 1] = cfma(a[u], ldc(V.v + j + u), acc[u & 1]);
            }
            for (; j < j1; ++j) {
              const bool up = j > i;
              double2 a0 = up ? ldc(T + j + (int64_t)i * lda) : ldc(T + i + (int64_t)j * lda);
              a0.y = cond_flip(a0.y, up);
              acc[0] = cfma(a0, ldc(V.v + j), acc[0]);
            }
            const double2 sum = make_double2(acc[0].x + acc[1].x, acc[0].y + acc[1].y);
            if (nseg == 1) {
              if (row < r1) {
                const double2 wi = cmul(tau, sum);
                V.w[i] = wi;
                const double2 vi = ldc(V.v + i);
                pr = fma(wi.x, vi.x, fma(wi.y, vi.y, pr));
                pi = fma(wi.x, vi.y, fma(-wi.y, vi.x, pi));
              }
            } else {
              hpart[sg * (G * 32) + g0 * 32 + lane] = sum;
            }
          }
          if (nseg > 1) {
            __syncthreads();
            for (int rl = tid; rl < r1 - r0; rl += CNT) {
              double2 sum = hpart[rl];
              for (int sg = 1; sg < nseg; ++sg) {
                const double2 q = hpart[sg * (G * 32) + rl];
                sum.x += q.x;
                sum.y += q.y;
              }
              const int i = r0 + rl;
              const double2 wi = cmul(tau, sum);
              V.w[i] = wi;
              const double2 vi = ldc(V.v + i);
              pr = fma(wi.x, vi.x, fma(wi.y, vi.y, pr));
              pi = fma(wi.x, vi.y, fma(-wi.y, vi.x, pi));
            }
          }
        }
        R.sum2(cl, pr, pi);   // its barrier also publishes w
        const double2 al = cmul(make_double2(-0.5 * tau.x, -0.5 * tau.y), make_double2(pr, pi));
        for (int i = gt; i < m; i += GT) V.w[i] = cfma(al, ldc(V.v + i), ldc(V.w + i));
        cl.sync();
        tri_update<1>(A + (k + 1) + (int64_t)(k + 1) * lda, lda, m, V.v, V.w, gt, GT);
        cl.sync();
        if (lead) x[0] = make_double2(beta, 0.0);
      } else {
        cl.sync();
        if (lead) A[(k + 1) + (int64_t)(k + 1) * lda].y = 0.0;
        cl.sync();
      }
    }
    if (lead) V.d[n - 1] = ldc(A + (n - 1) + (int64_t)(n - 1) * lda).x;
    cl.sync();

    // ------------------------------------------------------- tridiagonal eigenvalues
    // Every CTA copies the tridiagonal into its shared memory and derives the
    // same Gershgorin bounds.
    double lo = 1e300, hi = -1e300, emax = 0.0;
    for (int i = tid; i < n; i += CNT) {
      const double di = ldc(V.d + i);
      const double e2i = (i < n - 1) ? ldc(V.e2 + i) : 0.0;
      sd[i] = di;
      se2[i] = e2i;
      sd32[i] = (float)di;
      se232[i] = (float)e2i;
    }
    __syncthreads();
    for (int i = tid; i < n; i += CNT) {
      const double ea = (i > 0) ? sqrt(se2[i - 1]) : 0.0;
      const double eb = (i < n - 1) ? sqrt(se2[i]) : 0.0;
      lo = fmin(lo, sd[i] - ea - eb);
      hi = fmax(hi, sd[i] + ea + eb);
      if (i < n - 1) emax = fmax(emax, se2[i]);
    }
    for (int o = 16; o > 0; o >>= 1) {
      lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
      hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
      emax = fmax(emax, __shfl_xor_sync(0xffffffffu, emax, o));
    }
    if ((tid & 31) == 0) {
      red_warp[tid >> 5] = lo;
      red_warp[CNW + (tid >> 5)] = hi;
      red_warp[2 * CNW + (tid >> 5)] = emax;
    }
    __syncthreads();
    lo = red_warp[0];
    hi = red_warp[CNW];
    emax = red_warp[2 * CNW];
    for (int w = 1; w < CNW; ++w) {
      lo = fmin(lo, red_warp[w]);
      hi = fmax(hi, red_warp[CNW + w]);
      emax = fmax(emax, red_warp[2 * CNW + w]);
    }
    const skn_sturm::Bounds Bd = skn_sturm::make_bounds(lo, hi, emax, n);
    for (int j = gt; j < n; j += GT) eig[eig_off[p] + j] = skn_sturm::eigenvalue(sd, se2, sd32, se232, n, j, Bd);
    if (lead) status[p] = SKN_OK;
    cl.sync();   // the next problem reuses the cluster's vectors and shared memory
  }
}

size_t dyn_smem_bytes(int max_n) {
  const size_t b = (size_t)24 * (size_t)max_n;
  return b > (size_t)SMEM_FLOOR ? b : (size_t)SMEM_FLOOR;
}

// Clusters of `cluster` CTAs that fit on the device at once (capped at n_prob).
// The attributes are set to the same values on every call, so concurrent
// callers cannot undo each other.
cudaError_t cluster_config(int cluster, int n_prob, int max_n, int* clusters) {
  cudaError_t e = cudaFuncSetAttribute(k_eigh_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)dyn_smem_bytes(LARGE_MAX_N));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_eigh_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)cluster, 1, 1);
  cfg.blockDim = dim3(CNT, 1, 1);
  cfg.dynamicSmemBytes = dyn_smem_bytes(max_n);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int active = 0;
  e = cudaOccupancyMaxActiveClusters(&active, k_eigh_cluster, &cfg);
  if (e != cudaSuccess) return e;
  *clusters = active < n_prob ? active : n_prob;
  return cudaSuccess;
}

}  // namespace

extern "C" int skn_eigh_large_scratch_bytes(int n_prob, int max_n, int cluster, int64_t* bytes) {
  if (!bytes || n_prob < 0 || max_n < 0 || cluster < 1 || cluster > MAX_CLUSTER) return SKN_ERR_ARG;
  if (max_n > LARGE_MAX_N) return SKN_ERR_CAPACITY;
  const int mn = max_n < 1 ? 1 : max_n;
  int clusters = 0;
  if (cluster_config(cluster, n_prob > 0 ? n_prob : 1, mn, &clusters) != cudaSuccess) return SKN_ERR_CUDA;
  if (clusters < 1) return SKN_ERR_CAPACITY;
  *bytes = (int64_t)clusters * cluster_stride(mn) * (int64_t)sizeof(double);
  return SKN_OK;
}

extern "C" int skn_eigh_gen_large(int n_prob, const int32_t* n, const int64_t* hs_off, const int64_t* eig_off,
                                  const int32_t* order, double* H, double* S, double* eig, int32_t* status,
                                  int32_t* work_counter, double* scratch, int64_t scratch_bytes, int max_n,
                                  int cluster, cudaStream_t stream) {
  if (n_prob < 0 || max_n < 0 || cluster < 1 || cluster > MAX_CLUSTER) return SKN_ERR_ARG;
  if (n_prob == 0) return SKN_OK;
  if (!n || !hs_off || !eig_off || !order || !H || !S || !eig || !status || !work_counter || !scratch)
    return SKN_ERR_ARG;
  if (max_n > LARGE_MAX_N) return SKN_ERR_CAPACITY;
  const int mn = max_n < 1 ? 1 : max_n;
  int clusters = 0;
  if (cluster_config(cluster, n_prob, mn, &clusters) != cudaSuccess) return SKN_ERR_CUDA;
  if (clusters < 1) return SKN_ERR_CAPACITY;
  const int64_t need = (int64_t)clusters * cluster_stride(mn) * (int64_t)sizeof(double);
  if (scratch_bytes < need) return SKN_ERR_CAPACITY;
  if ((reinterpret_cast<uintptr_t>(scratch) & 15) != 0 || (reinterpret_cast<uintptr_t>(H) & 15) != 0 ||
      (reinterpret_cast<uintptr_t>(S) & 15) != 0)
    return SKN_ERR_ARG;   // complex elements are read as 16-byte vectors
  if (cudaMemsetAsync(work_counter, 0, sizeof(int32_t), stream) != cudaSuccess) return SKN_ERR_CUDA;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(clusters * cluster), 1, 1);
  cfg.blockDim = dim3(CNT, 1, 1);
  cfg.dynamicSmemBytes = dyn_smem_bytes(mn);
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)cluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const cudaError_t e = cudaLaunchKernelEx(&cfg, k_eigh_cluster, n_prob, n, hs_off, eig_off, order, (double2*)H,
                                           (double2*)S, eig, status, work_counter, scratch, mn);
  return e == cudaSuccess ? SKN_OK : SKN_ERR_CUDA;
}
