// Generalized Hermitian eigenvalues of large problems, blocked and spread over the whole GPU.
//
// For a group of problems of one size n (the k-points of one large structure) the host issues one
// sequence of kernel launches; every launch covers all problems of the group, and within a launch
// the CTAs of one problem work on tiles or row chunks of it, so every SM works on every step:
//   1. unit diagonal for all-zero rows (eighb's aux option, slakonet/utils.py:741-747);
//   2. Cholesky S = L L^H, right-looking, NB-column panels: the NB x NB diagonal block in one warp,
//      the panel's rows solved in parallel, then one tiled rank-NB update of the trailing triangle;
//   3. reduction to C = L^-1 H L^-H in LAPACK zhegst order (lower, itype 1) per panel: zhegs2 on the
//      diagonal block, A21 L11^-H, -1/2 L21 A11, a tiled rank-2NB update A22 -= A21 L21^H + L21 A21^H,
//      -1/2 L21 A11.  The last step of each panel, A21 <- L22^-1 A21, touches nothing later panels
//      read, so the solves of all panels are deferred and run together as one blocked forward
//      substitution (per 32-row chunk: a diagonal solve, then a tiled GEMM update of the rows below);
//   4. Householder tridiagonalisation in LAPACK zlatrd order: per column a column update from the
//      panel's earlier reflectors, the reflector, a tiled Hermitian matrix-vector product with the
//      trailing matrix as it stood at the panel's start, the panel corrections, and w; per panel one
//      tiled rank-2NB update A22 -= V W^H + W V^H;
//   5. eigenvalues of the tridiagonal by Sturm counts and Newton (sturm.cuh), one thread each.
// The reference calls torch.linalg.cholesky / solve / eigh per k (slakonet/utils.py:749-783,
// slakonet/main.py:174).
//
// Every partial sum that crosses CTAs (hemv tiles, norms, dot products) is written to its own slot
// and summed in a fixed order by the next launch: no floating-point atomics, so a problem's results
// do not depend on the other problems of its group or on how the group is scheduled.
//
// GB300 notes.  FP64 is the bound (about 1.25 TFLOP/s per GPU; a warp FP64 instruction costs the
// same with 1 or 32 lanes), so the O(n^3) work sits in tile kernels whose threads each hold a 4x4
// block of complex accumulators fed from shared memory (8 shared loads per 64 FMAs), and the
// matrix-vector product reads each 64x64 tile once for both of its products.  R = true runs the same
// code on the real parts only (problems whose H(k), S(k) are exactly real).
#include <cuda_bf16.h>

#include "exact_round.cuh"
#include "skn_common.cuh"
#include "sturm.cuh"

namespace {

constexpr int NB = 32;                 // panel width
constexpr int TS = 64;                 // tile edge of the product kernels
constexpr int KC = 16;                 // panel columns staged per pass of the tile kernels
constexpr int RC = 64;                 // rows per CTA of the row-parallel kernels (many CTAs at mid sizes)
constexpr int WIDE_MAX_N = 32768;
constexpr int TLD = TS + 1;            // leading dimension of the staged hemv tile
constexpr int TCS = 7;                 // integer slices per operand row in the tensor-core update

SKN_DEVINL int cdiv_d(int a, int b) { return (a + b - 1) / b; }
// Rows of each slice array of the tensor-core update: n rounded up to whole 128-row tiles, so a tile's block
// of rows never ends past the array.
__host__ __device__ inline int64_t tc_rows(int n) { return ((int64_t)n + 127) / 128 * 128; }
// Element index of (row r, column k) in a slice array with kp columns, in the tensor cores' K-major
// core-matrix order: 8-row groups of kp * 8 elements, each a run of 8 x 8 core matrices (8 rows x 16 bytes)
// along K.  A 128-row (or 32-row) block starting at a multiple of 8 is one contiguous run in exactly the
// order the MMA's shared-memory descriptor reads (LBO 128 bytes, SBO kp * 16 bytes), so it is staged by a
// single bulk copy.
SKN_DEVINL int64_t tc_idx(int r, int k, int kp) {
  return (int64_t)(r >> 3) * (8 * kp) + (k >> 3) * 64 + (r & 7) * 8 + (k & 7);
}
inline int cdiv(int a, int b) { return (a + b - 1) / b; }

// ------------------------------------------------------------------ arithmetic (R: real parts only)
template <bool R> SKN_DEVINL double2 zld(const double2* p) {
  if constexpr (R) return make_double2(p->x, 0.0); else return *p;
}
template <bool R> SKN_DEVINL void zst(double2* p, double2 v) {
  if constexpr (R) p->x = v.x; else *p = v;
}
template <bool R> SKN_DEVINL double2 zfma(double2 a, double2 b, double2 c) {        // c + a b
  if constexpr (R) { c.x = fma(a.x, b.x, c.x); return c; } else return cfma(a, b, c);
}
template <bool R> SKN_DEVINL double2 zfma_cj(double2 a, double2 b, double2 c) {     // c + a conj(b)
  if constexpr (R) { c.x = fma(a.x, b.x, c.x); return c; }
  c.x = fma(a.x, b.x, c.x);
  c.x = fma(a.y, b.y, c.x);
  c.y = fma(a.y, b.x, c.y);
  c.y = fma(-a.x, b.y, c.y);
  return c;
}
template <bool R> SKN_DEVINL double2 zfma_cja(double2 a, double2 b, double2 c) {    // c + conj(a) b
  if constexpr (R) { c.x = fma(a.x, b.x, c.x); return c; } else return cfma_conj(a, b, c);
}
template <bool R> SKN_DEVINL double2 zfms(double2 a, double2 b, double2 c) {        // c - a b
  if constexpr (R) { c.x = fma(-a.x, b.x, c.x); return c; }
  c.x = fma(-a.x, b.x, c.x);
  c.x = fma(a.y, b.y, c.x);
  c.y = fma(-a.x, b.y, c.y);
  c.y = fma(-a.y, b.x, c.y);
  return c;
}
template <bool R> SKN_DEVINL double2 zfms_cj(double2 a, double2 b, double2 c) {     // c - a conj(b)
  if constexpr (R) { c.x = fma(-a.x, b.x, c.x); return c; } else return cfms_conj(a, b, c);
}
template <bool R> SKN_DEVINL double2 zmul(double2 a, double2 b) {
  if constexpr (R) return make_double2(a.x * b.x, 0.0); else return cmul(a, b);
}
template <bool R> SKN_DEVINL double2 zscal(double2 a, double s) {
  if constexpr (R) return make_double2(a.x * s, 0.0); else return cscale(a, s);
}
template <bool R> SKN_DEVINL double2 zsub(double2 a, double2 b) {
  return make_double2(a.x - b.x, R ? 0.0 : a.y - b.y);
}
template <bool R> SKN_DEVINL double2 zadd(double2 a, double2 b) {
  return make_double2(a.x + b.x, R ? 0.0 : a.y + b.y);
}
SKN_DEVINL double2 zconj(double2 a) { return make_double2(a.x, flip_sign(a.y)); }

// ------------------------------------------------------------------ scratch layout (per problem slot)
// All offsets in double2 units, each region 256-byte aligned.
struct Lay {
  int64_t W, v, y, Yp, r1, r2, r3, sc, d, e2, rd, d32, e232, flg, tcs, tce, stride;
};
__host__ __device__ inline int64_t take(int64_t& o, int64_t cnt) {
  const int64_t r = o;
  o += (cnt + 15) / 16 * 16;
  return r;
}
__host__ __device__ inline Lay layout(int n) {
  const int64_t nt = (n + TS - 1) / TS, nch = (n + RC - 1) / RC;
  Lay L;
  int64_t o = 0;
  L.W = take(o, (int64_t)NB * n);        // W panel, column q at W + q*n (global row index)
  L.v = take(o, n);                      // Householder vector, A22-relative
  L.y = take(o, n);                      // hemv result, A22-relative
  L.Yp = take(o, nt * n);                // hemv partial sums: slot s at Yp + s*n
  L.r1 = take(o, nch);                   // norm partials (x)
  L.r2 = take(o, nch * 2 * NB);          // dot-product partials: chunk c at r2 + c*2NB
  L.r3 = take(o, nch);                   // w^H v partials
  L.sc = take(o, 16);                    // scalars
  L.d = take(o, (n + 1) / 2);
  L.e2 = take(o, (n + 1) / 2);
  L.rd = take(o, (n + 1) / 2);
  L.d32 = take(o, (n + 3) / 4);
  L.e232 = take(o, (n + 3) / 4);
  L.flg = take(o, (2 * (int64_t)n + 3) / 4);
  L.tcs = take(o, (int64_t)3 * TCS * tc_rows(n) * 128 * 2 / 16);   // bf16 slices of the tensor-core update
  L.tce = take(o, ((int64_t)n + 3) / 4);                    // their row exponents
  L.stride = o;
  return L;
}

struct WS {
  double2 *W, *v, *y, *Yp, *r1, *r2, *r3, *sc;
  double *d, *e2, *rd;
  float *d32, *e232;
  int* flg;
  uint16_t* tcs;   // bf16 slices: [form][TCS][tc_rows(n) x KP in tc_idx order], form 0 A, 1 A' (complex), 2 B
  int* tce;        // row exponents of the sliced rows
};

// What every launch needs: the group and its buffers.
struct Grp {
  int n, n_prob;
  const int32_t* prob;     // [n_prob] problem index of each slot
  const int32_t* nvec;     // [*] orbitals per problem (must equal n)
  const int64_t* hs_off;   // [*] element offset of a problem's H and S
  const int64_t* eig_off;  // [*] offset of its eigenvalues
  double2* H;
  double2* S;
  double* eig;
  int32_t* status;
  double2* scratch;
};

SKN_DEVINL WS ws_of(const Grp& G, int g) {
  const Lay L = layout(G.n);
  double2* b = G.scratch + (int64_t)g * L.stride;
  WS w;
  w.W = b + L.W; w.v = b + L.v; w.y = b + L.y; w.Yp = b + L.Yp;
  w.r1 = b + L.r1; w.r2 = b + L.r2; w.r3 = b + L.r3; w.sc = b + L.sc;
  w.d = reinterpret_cast<double*>(b + L.d);
  w.e2 = reinterpret_cast<double*>(b + L.e2);
  w.rd = reinterpret_cast<double*>(b + L.rd);
  w.d32 = reinterpret_cast<float*>(b + L.d32);
  w.e232 = reinterpret_cast<float*>(b + L.e232);
  w.flg = reinterpret_cast<int*>(b + L.flg);
  w.tcs = reinterpret_cast<uint16_t*>(b + L.tcs);
  w.tce = reinterpret_cast<int*>(b + L.tce);
  return w;
}

// A matrix operand of the tile kernels: src 0 = H, 1 = S (problem p), 2 = the W panel (slot g);
// `off` is the element offset of its (0, 0) entry; every operand has leading dimension n.
struct Mat {
  int src;
  int64_t off;
};
SKN_DEVINL double2* mat_ptr(const Grp& G, int g, int p, Mat M) {
  if (M.src == 2) return ws_of(G, g).W + M.off;
  return (M.src == 0 ? G.H : G.S) + G.hs_off[p] + M.off;
}

// Lower-triangle tile index t -> (I, J), I >= J.
SKN_DEVINL void tile_ij(int t, int& I, int& J) {
  int i = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
  while (i > 0 && i * (i + 1) / 2 > t) --i;
  while ((i + 1) * (i + 2) / 2 <= t) ++i;
  I = i;
  J = t - i * (i + 1) / 2;
}

SKN_DEVINL bool live(const Grp& G, int p) { return G.status[p] == SKN_OK; }

// Sum of count values base[c * stride] by one warp: lane l adds c = l, l + 32, ... in order, then a fixed
// butterfly; every lane returns the same bits, whatever the launch.
template <bool R>
SKN_DEVINL double2 warp_chunk_sum(const double2* base, int64_t stride, int count) {
  const int lane = threadIdx.x & 31;
  double2 s = make_double2(0.0, 0.0);
  for (int c = lane; c < count; c += 32) s = zadd<R>(s, zld<R>(base + (int64_t)c * stride));
  for (int o = 16; o > 0; o >>= 1) {
    s.x += __shfl_xor_sync(0xffffffffu, s.x, o);
    if constexpr (!R) s.y += __shfl_xor_sync(0xffffffffu, s.y, o);
  }
  return s;
}

// ------------------------------------------------------------------ set-up
// Status per problem (size check) and cleared zero-row flags.
__global__ void __launch_bounds__(256) k_init(Grp G) {
  const int g = blockIdx.y, p = G.prob[g];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const bool ok = G.nvec[p] == G.n && G.hs_off[p] >= 0 && G.eig_off[p] >= 0;
    G.status[p] = ok ? SKN_OK : SKN_ERR_CAPACITY;
  }
  const int i = blockIdx.x * 256 + threadIdx.x;
  if (i < 2 * G.n) ws_of(G, g).flg[i] = 0;
}

// Marks rows with a nonzero entry: thread per row over a 256-column chunk of the lower triangle;
// an entry (i, j) marks row i and (as the conjugate entry (j, i)) row j.
template <bool R>
__global__ void __launch_bounds__(256) k_zscan(Grp G) {
  const int g = blockIdx.z >> 1, which = blockIdx.z & 1, p = G.prob[g];
  if (!live(G, p)) return;
  const int n = G.n;
  const int i = blockIdx.x * 256 + threadIdx.x;
  const int c0 = blockIdx.y * 256;
  if (c0 > blockIdx.x * 256 + 255) return;      // the chunk lies above the diagonal
  const double2* A = (which ? G.S : G.H) + G.hs_off[p];
  int* flg = ws_of(G, g).flg + which * n;
  bool row_nz = false;
  const int c1 = min(c0 + 256, n);
  for (int j = c0; j < c1; ++j) {
    bool nz = false;
    if (i < n && j <= i) {
      const double2 a = A[i + (int64_t)j * n];
      nz = !(is_zero_bits(a.x) && is_zero_bits(a.y));
    }
    row_nz |= nz;
    if (__any_sync(0xffffffffu, nz) && (threadIdx.x & 31) == 0) flg[j] = 1;
  }
  if (row_nz) flg[i] = 1;
}

template <bool R>
__global__ void __launch_bounds__(256) k_zfix(Grp G) {
  const int g = blockIdx.y >> 1, which = blockIdx.y & 1, p = G.prob[g];
  if (!live(G, p)) return;
  const int n = G.n, i = blockIdx.x * 256 + threadIdx.x;
  if (i >= n) return;
  if (ws_of(G, g).flg[which * n + i] == 0) ((which ? G.S : G.H) + G.hs_off[p])[i + (int64_t)i * n].x += 1.0;
}

// ------------------------------------------------------------------ Cholesky
// Unblocked Cholesky of the w x w diagonal block at (c0, c0) of S by one warp (lane = row).
template <bool R>
__global__ void __launch_bounds__(32) k_potrf(Grp G, int c0, int w) {
  const int g = blockIdx.x, p = G.prob[g];
  if (!live(G, p)) return;
  const int n = G.n, lane = threadIdx.x;
  __shared__ double2 Lt[NB * (NB + 1)];
  double2* A11 = G.S + G.hs_off[p] + c0 + (int64_t)c0 * n;
  double* rd = ws_of(G, g).rd;
  for (int e = lane; e < w * w; e += 32) {
    const int i = e % w, j = e / w;
    if (i >= j) Lt[i + j * (NB + 1)] = zld<R>(A11 + i + (int64_t)j * n);
  }
  __syncwarp();
  int bad = 0;
  for (int k = 0; k < w; ++k) {
    const double a = Lt[k + k * (NB + 1)].x;
    const bool ok = (a > 0.0) && is_finite_bits(a);
    bad |= ok ? 0 : 1;
    const double dk = ok ? sqrt(a) : 1.0;
    const double r = 1.0 / dk;
    __syncwarp();
    if (lane == k) {
      Lt[k + k * (NB + 1)] = make_double2(dk, 0.0);
      rd[c0 + k] = r;
    }
    double2 lik = make_double2(0.0, 0.0);
    if (lane > k && lane < w) {
      lik = zscal<R>(Lt[lane + k * (NB + 1)], r);
      Lt[lane + k * (NB + 1)] = lik;
    }
    __syncwarp();
    if (lane > k && lane < w)
      for (int j = k + 1; j <= lane; ++j)
        Lt[lane + j * (NB + 1)] = zfms_cj<R>(lik, Lt[j + k * (NB + 1)], Lt[lane + j * (NB + 1)]);
    __syncwarp();
  }
  for (int e = lane; e < w * w; e += 32) {
    const int i = e % w, j = e / w;
    if (i >= j) zst<R>(A11 + i + (int64_t)j * n, Lt[i + j * (NB + 1)]);
  }
  if (bad && lane == 0) G.status[p] = SKN_ERR_NOT_SPD;
}

// A21 <- A21 L11^-H for the m rows below the panel at c0 (A = H or S, L11 from S), thread per row.
template <bool R>
__global__ void __launch_bounds__(RC) k_trsm_right(Grp G, int which, int c0, int m) {
  const int g = blockIdx.y, p = G.prob[g];
  if (!live(G, p)) return;
  const int n = G.n;
  __shared__ double2 Lt[NB * (NB + 1)];
  __shared__ double rds[NB];
  const double2* L11 = G.S + G.hs_off[p] + c0 + (int64_t)c0 * n;
  for (int e = threadIdx.x; e < NB * NB; e += RC) {
    const int i = e % NB, j = e / NB;
    if (i >= j) Lt[i + j * (NB + 1)] = zld<R>(L11 + i + (int64_t)j * n);
  }
  if (threadIdx.x < NB) rds[threadIdx.x] = ws_of(G, g).rd[c0 + threadIdx.x];
  __syncthreads();
  const int r = blockIdx.x * RC + threadIdx.x;
  if (r >= m) return;
  double2* row = (which ? G.S : G.H) + G.hs_off[p] + (c0 + NB + r) + (int64_t)c0 * n;
  double2 x[NB];
#pragma unroll
  for (int j = 0; j < NB; ++j) x[j] = zld<R>(row + (int64_t)j * n);
#pragma unroll
  for (int j = 0; j < NB; ++j) {
    double2 a0 = x[j], a1 = make_double2(0.0, 0.0);
#pragma unroll
    for (int k = 0; k < j; ++k) {
      if (k & 1) a1 = zfms_cj<R>(x[k], Lt[j + k * (NB + 1)], a1);
      else a0 = zfms_cj<R>(x[k], Lt[j + k * (NB + 1)], a0);
    }
    x[j] = zscal<R>(zadd<R>(a0, a1), rds[j]);
  }
#pragma unroll
  for (int j = 0; j < NB; ++j) zst<R>(row + (int64_t)j * n, x[j]);
}

// C -= P P^H (MODE 0) or C -= P Q^H + Q P^H (MODE 1) on the lower triangle of the m x m matrix C,
// P and Q m x K (K <= NB).  One CTA of (T/4)^2 threads per T x T tile; each thread a 4x4 block of
// accumulators.  T = 64 for large trailing matrices, 32 when 64-wide tiles would not fill the GPU twice.
template <bool R, int MODE, int T>
__global__ void __launch_bounds__((T / 4) * (T / 4)) k_rank2k(Grp G, Mat Cm, int m, Mat Pm, Mat Qm, int K) {
  constexpr int NTH = (T / 4) * (T / 4);
  const int g = blockIdx.y, p = G.prob[g];
  if (!live(G, p)) return;
  const int n = G.n;
  int I, J;
  tile_ij(blockIdx.x, I, J);
  extern __shared__ double2 smr[];
  double2* sPI = smr;
  double2* sQJ = smr + KC * T;             // MODE 0: P rows of tile J
  double2* sQI = smr + 2 * KC * T;
  double2* sPJ = smr + 3 * KC * T;
  double2* C = mat_ptr(G, g, p, Cm);
  const double2* P = mat_ptr(G, g, p, Pm);
  const double2* Q = MODE ? mat_ptr(G, g, p, Qm) : P;
  const int tid = threadIdx.x, tr = tid % (T / 4), tc = tid / (T / 4);
  double2 acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = make_double2(0.0, 0.0);
  for (int k0 = 0; k0 < K; k0 += KC) {
    for (int e = tid; e < KC * T; e += NTH) {
      const int r = e % T, k = e / T, kk = k0 + k;
      const int gi = I * T + r, gj = J * T + r;
      const bool okI = gi < m && kk < K, okJ = gj < m && kk < K;
      const double2 z = make_double2(0.0, 0.0);
      sPI[k * T + r] = okI ? zld<R>(P + gi + (int64_t)kk * n) : z;
      sQJ[k * T + r] = okJ ? zld<R>(Q + gj + (int64_t)kk * n) : z;
      if (MODE) {
        sQI[k * T + r] = okI ? zld<R>(Q + gi + (int64_t)kk * n) : z;
        sPJ[k * T + r] = okJ ? zld<R>(P + gj + (int64_t)kk * n) : z;
      }
    }
    __syncthreads();
#pragma unroll 2
    for (int k = 0; k < KC; ++k) {
      double2 a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) a[u] = sPI[k * T + tr * 4 + u];
#pragma unroll
      for (int v = 0; v < 4; ++v) b[v] = sQJ[k * T + tc * 4 + v];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = zfma_cj<R>(a[u], b[v], acc[u][v]);
      if (MODE) {
#pragma unroll
        for (int u = 0; u < 4; ++u) a[u] = sQI[k * T + tr * 4 + u];
#pragma unroll
        for (int v = 0; v < 4; ++v) b[v] = sPJ[k * T + tc * 4 + v];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int v = 0; v < 4; ++v) acc[u][v] = zfma_cj<R>(a[u], b[v], acc[u][v]);
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const int c = J * T + tc * 4 + v;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int r = I * T + tr * 4 + u;
      if (r < m && c < m && r >= c) {
        double2* t = C + r + (int64_t)c * n;
        double2 val = zsub<R>(zld<R>(t), acc[u][v]);
        if (r == c) val.y = 0.0;
        zst<R>(t, val);
      }
    }
  }
}

// ------------------------------------------------------------------ rank-2k on the tensor cores
// The same update as k_rank2k, C -= P Q^H + Q P^H (MODE 1) or C -= P P^H (MODE 0), computed on the bf16
// tensor cores by error-free splitting (Ozaki, Ogita and Oishi, Numer. Algorithms 59, 2012).  In real form
// the complex update is two real products with a 4K-wide inner dimension KP = 128:
//   C_r -= A B^T,  C_i -= A' B^T,  A = [Pr Pi Qr Qi],  A' = [Pi -Pr Qi -Qr],  B = [Qr Qi Pr Pi]
// (MODE 0: A = [Pr Pi 0 0], A' = [Pi -Pr 0 0], B = [Pr Pi 0 0]); a real problem needs one product with
// KP = 64, A = [P Q], B = [Q P] (MODE 0: [P 0], [P 0]).  Every row of A, A' and B holds the same values, so
// one exponent e_r per row serves all three: x = 2^e_r sum_s d_s 2^(-7(s+1)) with TCS integer digits
// d_s (rounded to nearest, |d_0| <= 128, later |d_s| <= 64), each exact in bf16.  A slice product is an
// integer below 2^14 and a K = 128 sum below 2^21, so all slice pairs with the same level s + t (at most
// TCS = 7 of them) accumulate exactly in one FP32 TMEM accumulator (below 2^24).  The levels are combined
// exactly in two int64 halves and rounded once to FP64.  With 7 slices of 7 bits the dropped pairs
// (s + t >= 7) and digits lie near 2^-49 of each row's scale.

SKN_DEVINL uint32_t smem_u32(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// Shared-memory matrix descriptor: no swizzle, K-major core matrices (8 rows x 16 bytes), LBO = 128 bytes
// between core matrices along K, sbo bytes between 8-row groups.
SKN_DEVINL uint64_t tc_desc(uint32_t addr, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)((128u >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor, kind::f16: D F32, A and B BF16, both K-major, M = 128, N = 32.
constexpr uint32_t TC_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(32 >> 3) << 17) |
                              ((uint32_t)(128 >> 4) << 24);

SKN_DEVINL void tc_mma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t"
      "}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(TC_IDESC), "r"(accumulate));
}

constexpr long long TC_WAIT_LIMIT = 1LL << 26;    // mbarrier polls before giving up

SKN_DEVINL bool tc_wait(uint32_t bar, uint32_t parity) {
  for (long long it = 0; it < TC_WAIT_LIMIT; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t"
        "}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity));
    if (done) return true;
  }
  return false;
}

SKN_DEVINL uint16_t bf16_bits(double d) { return __bfloat16_as_ushort(__double2bfloat16(d)); }

// Slices of the m rows of the panel update (one warp per row; lane l holds column l of each K block).
template <bool R, int MODE>
__global__ void __launch_bounds__(256) k_r2k_split(Grp G, Mat Pm, Mat Qm, int m, int K) {
  constexpr int KP = R ? 64 : 128, NSEC = KP / 32;
  const int g = blockIdx.y, p = G.prob[g];
  if (!live(G, p)) return;
  const int n = G.n, lane = threadIdx.x & 31;
  const int r = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (r >= m) return;
  const WS w = ws_of(G, g);
  const double2* P = mat_ptr(G, g, p, Pm);
  const double2* Q = MODE ? mat_ptr(G, g, p, Qm) : P;
  // x[0..NSEC): complex [Pr, Pi, Qr, Qi], real [P, Q]; zero beyond K, and the Q part in MODE 0
  double x[4] = {0.0, 0.0, 0.0, 0.0};
  if (lane < K) {
    const double2 pv = zld<R>(P + r + (int64_t)lane * n);
    const double2 qv = MODE ? zld<R>(Q + r + (int64_t)lane * n) : make_double2(0.0, 0.0);
    if constexpr (R) {
      x[0] = pv.x;
      x[1] = qv.x;
    } else {
      x[0] = pv.x;
      x[1] = pv.y;
      x[2] = qv.x;
      x[3] = qv.y;
    }
  }
  double amax = 0.0;
#pragma unroll
  for (int i = 0; i < NSEC; ++i) amax = fmax(amax, fabs(x[i]));
  for (int o = 16; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
  int ex = 0;
  if (amax > 0.0) frexp(amax, &ex);                 // amax = f 2^ex, f in [0.5, 1): |x| 2^-ex < 1
  if (lane == 0) w.tce[r] = ex;
  double v[4];
#pragma unroll
  for (int i = 0; i < NSEC; ++i) v[i] = ldexp(x[i], -ex);   // exact
  const int64_t np = tc_rows(n);
  uint16_t* base = w.tcs;
  int64_t ix[NSEC];                                 // this lane's columns of row r: lane, 32 + lane, ...
#pragma unroll
  for (int i = 0; i < NSEC; ++i) ix[i] = tc_idx(r, 32 * i + lane, KP);
  for (int sl = 0; sl < TCS; ++sl) {
    double dgt[4];
#pragma unroll
    for (int i = 0; i < NSEC; ++i) {
      v[i] *= 128.0;                                // exact
      dgt[i] = rint(v[i]);                          // |dgt| <= 128, then <= 64
      v[i] -= dgt[i];                               // exact remainder
    }
    uint16_t* A = base + (int64_t)(0 * TCS + sl) * np * KP;
    uint16_t* B = base + (int64_t)((R ? 1 : 2) * TCS + sl) * np * KP;
    if constexpr (R) {
      A[ix[0]] = bf16_bits(dgt[0]);
      A[ix[1]] = bf16_bits(dgt[1]);
      B[ix[0]] = bf16_bits(MODE ? dgt[1] : dgt[0]);
      B[ix[1]] = bf16_bits(MODE ? dgt[0] : 0.0);
    } else {
      uint16_t* A2 = base + (int64_t)(1 * TCS + sl) * np * KP;
      A[ix[0]] = bf16_bits(dgt[0]);
      A[ix[1]] = bf16_bits(dgt[1]);
      A[ix[2]] = bf16_bits(dgt[2]);
      A[ix[3]] = bf16_bits(dgt[3]);
      A2[ix[0]] = bf16_bits(dgt[1]);
      A2[ix[1]] = bf16_bits(-dgt[0]);
      A2[ix[2]] = bf16_bits(dgt[3]);
      A2[ix[3]] = bf16_bits(-dgt[2]);
      if (MODE) {
        B[ix[0]] = bf16_bits(dgt[2]);
        B[ix[1]] = bf16_bits(dgt[3]);
        B[ix[2]] = bf16_bits(dgt[0]);
        B[ix[3]] = bf16_bits(dgt[1]);
      } else {
        B[ix[0]] = bf16_bits(dgt[0]);
        B[ix[1]] = bf16_bits(dgt[1]);
        B[ix[2]] = bf16_bits(0.0);
        B[ix[3]] = bf16_bits(0.0);
      }
    }
  }
}

// Bulk copy of `bytes` contiguous bytes from global to this CTA's shared memory, completing on `bar`
// (complete_tx); both addresses 16-byte aligned, bytes a multiple of 16.
SKN_DEVINL void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(dst), "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}
SKN_DEVINL void bar_expect(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// One CTA (4 warps) per 128 x 32 tile of C's lower triangle.  Thread 0 runs a two-stage pipeline: the TCS
// slices of the tile's 32 B rows and the first two slices of its 128 A rows (and A' for complex problems)
// arrive by bulk copies, each one contiguous block of the slice arrays (their tc_idx order is the MMA's
// shared-memory layout); for each A slice s, once its copy has landed, thread 0 issues the MMAs of every
// pair (s, t) with s + t < TCS into the level accumulator s + t in TMEM and commits them to that stage's
// mbarrier, and when those MMAs are done it refills the stage with slice s + 2, so copies overlap the MMAs
// of the other stage.  All waits are bounded.  The epilogue reads each level with tcgen05.ld, combines the
// levels exactly in int64, rounds once to FP64 with the scale 2^(e_row + e_col) (exact_to_double) and
// subtracts from C.  A wait that runs out marks
// the problem's status SKN_ERR_CUDA and leaves its C tile unchanged; thread 0 then still waits (bounded)
// for every copy and MMA it issued before the CTA frees its TMEM and exits.
template <bool R>
__global__ void __launch_bounds__(128) k_r2k_tc(Grp G, Mat Cm, int m) {
  constexpr int KP = R ? 64 : 128;
  constexpr uint32_t SBO = (KP / 8) * 128;         // bytes between 8-row groups of a staged tile
  constexpr int A_BYTES = 128 * KP * 2, B_BYTES = 32 * KP * 2;
  constexpr int NACC = R ? 1 : 2;                  // accumulators per level (C_r, C_i)
  constexpr uint32_t TMEM_COLS = R ? 256 : 512;    // TCS levels x NACC x 32 columns, rounded up
  const int g = blockIdx.y, p = G.prob[g];
  if (!live(G, p)) return;
  const int n = G.n;
  const int nJ = cdiv_d(m, 32);
  const int I = blockIdx.x / nJ, J = blockIdx.x % nJ;
  const int r0 = I * 128, c0 = J * 32;
  if (r0 + 127 < c0) return;                       // entirely above the diagonal
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sB = smem;                              // TCS tiles of 32 rows
  uint8_t* sA = smem + TCS * B_BYTES;              // 2 stages x NACC tiles of 128 rows
  // 0: B slices landed; 1, 2: stage 0 / 1 landed; 3, 4: the MMAs reading stage 0 / 1 are done
  __shared__ __align__(8) uint64_t bars[5];
  __shared__ uint32_t tmem_slot;
  __shared__ int s_fail;
  __shared__ int s_ce[32];
  const WS w = ws_of(G, g);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    s_fail = 0;
    for (int b = 0; b < 5; ++b) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[b])));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid < 32) s_ce[tid] = (c0 + tid < m) ? w.tce[c0 + tid] : 0;
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_slot;
  if (tid == 0) {
    const int64_t np = tc_rows(n);
    const uint16_t* slices = w.tcs;
    auto slice = [&](int f, int sl) { return slices + (int64_t)(f * TCS + sl) * np * KP; };
    const uint32_t bar_b = smem_u32(&bars[0]);
    const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
    auto load_stage = [&](int st, int sl) {
      const uint32_t bar = smem_u32(&bars[1 + st]);
      bar_expect(bar, NACC * A_BYTES);
      for (int f = 0; f < NACC; ++f)
        bulk_g2s(a0 + (uint32_t)((st * NACC + f) * A_BYTES), slice(f, sl) + (int64_t)r0 * KP, A_BYTES, bar);
    };
    bar_expect(bar_b, TCS * B_BYTES);
    for (int t = 0; t < TCS; ++t)
      bulk_g2s(b0 + (uint32_t)(t * B_BYTES), slice(R ? 1 : 2, t) + (int64_t)c0 * KP, B_BYTES, bar_b);
    load_stage(0, 0);
    load_stage(1, 1);
    // armed[b]: phases of mbarrier b armed (copies issued or MMAs committed) and not yet waited for
    int armed[5] = {1, 1, 1, 0, 0};
    int done[5] = {0, 0, 0, 0, 0};              // phases waited for
    bool ok = tc_wait(bar_b, 0);
    if (ok) done[0] = 1;
    for (int sl = 0; ok && sl < TCS; ++sl) {
      const int st = sl & 1;
      ok = tc_wait(smem_u32(&bars[1 + st]), (uint32_t)(done[1 + st] & 1));
      if (!ok) break;
      ++done[1 + st];
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t as = a0 + (uint32_t)(st * NACC * A_BYTES);
      for (int t = 0; t + sl < TCS; ++t) {
        const uint32_t col = (uint32_t)((sl + t) * NACC * 32);
#pragma unroll
        for (int kk = 0; kk < KP / 16; ++kk) {
          const uint32_t acc = (sl > 0 || kk > 0) ? 1u : 0u;
          const uint64_t bd = tc_desc(b0 + t * B_BYTES + kk * 256, SBO);
          tc_mma(tmem + col, tc_desc(as + kk * 256, SBO), bd, acc);
          if (NACC == 2) tc_mma(tmem + col + 32, tc_desc(as + A_BYTES + kk * 256, SBO), bd, acc);
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(&bars[3 + st])));
      ++armed[3 + st];
      if (sl + 2 < TCS) {                         // refill this stage once its MMAs have read it
        ok = tc_wait(smem_u32(&bars[3 + st]), (uint32_t)(done[3 + st] & 1));
        if (!ok) break;
        ++done[3 + st];
        load_stage(st, sl + 2);
        ++armed[1 + st];
      }
    }
    // every copy and MMA issued must have completed before the epilogue reads TMEM or the CTA exits
    for (int b = 0; b < 5; ++b)
      while (done[b] < armed[b]) {
        if (!tc_wait(smem_u32(&bars[b]), (uint32_t)(done[b] & 1))) {
          ok = false;
          break;
        }
        ++done[b];
      }
    if (!ok) s_fail = 1;
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (!s_fail) {
    const int row = r0 + warp * 32 + lane;        // this thread's TMEM lane
    const int re = (row < m) ? w.tce[row] - 56 : 0;   // the level sums count units of 2^(e_row + e_col - 56)
    double2* C = mat_ptr(G, g, p, Cm);
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    for (int cb = 0; cb < 32; cb += 8) {
      long long hr[8], lr[8], hi[8], li[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) hr[q] = lr[q] = hi[q] = li[q] = 0;
#pragma unroll
      for (int L = 0; L < TCS; ++L) {
        uint32_t vr[8], vi[8];
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                     : "=r"(vr[0]), "=r"(vr[1]), "=r"(vr[2]), "=r"(vr[3]), "=r"(vr[4]), "=r"(vr[5]), "=r"(vr[6]),
                       "=r"(vr[7])
                     : "r"(lane_base + (uint32_t)(L * NACC * 32 + cb)));
        if (NACC == 2)
          asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                       : "=r"(vi[0]), "=r"(vi[1]), "=r"(vi[2]), "=r"(vi[3]), "=r"(vi[4]), "=r"(vi[5]), "=r"(vi[6]),
                         "=r"(vi[7])
                       : "r"(lane_base + (uint32_t)(L * NACC * 32 + 32 + cb)));
        asm volatile("tcgen05.wait::ld.sync.aligned;");
        const int sh = (L <= 3) ? 7 * (3 - L) : 7 * (6 - L);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const long long a = (long long)__float2int_rn(__uint_as_float(vr[q])) << sh;
          if (L <= 3) hr[q] += a; else lr[q] += a;
          if (NACC == 2) {
            const long long b = (long long)__float2int_rn(__uint_as_float(vi[q])) << sh;
            if (L <= 3) hi[q] += b; else li[q] += b;
          }
        }
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int col = c0 + cb + q;
        if (row < m && col < m && row >= col) {
          const int e = re + s_ce[cb + q];
          double2* t = C + row + (int64_t)col * n;
          double2 cv = zld<R>(t);
          cv.x -= exact_to_double(hr[q], lr[q], e);
          if (NACC == 2) cv.y = (row == col) ? 0.0 : cv.y - exact_to_double(hi[q], li[q], e);
          zst<R>(t, cv);
        }
      }
    }
  } else if (tid == 0) {
    G.status[p] = SKN_ERR_CUDA;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
}

// ------------------------------------------------------------------ reduction to standard form
// A11 <- L11^-1 A11 L11^-H on the w x w diagonal block at (c0, c0) by one warp: X = L^-1 A by
// columns, then C = L^-1 X^H (C is Hermitian), lane = column.
template <bool R>
__global__ void __launch_bounds__(32) k_hegs2(Grp G, int c0, int w) {
  const int g = blockIdx.x, p = G.prob[g];
  if (!live(G, p)) return;
  const int n = G.n, lane = threadIdx.x;
  __shared__ double2 Ls[NB * (NB + 1)], As[NB * (NB + 1)];
  __shared__ double rds[NB];
  double2* A11 = G.H + G.hs_off[p] + c0 + (int64_t)c0 * n;
  const double2* L11 = G.S + G.hs_off[p] + c0 + (int64_t)c0 * n;
  for (int e = lane; e < w * w; e += 32) {
    const int i = e % w, j = e / w;
    if (i >= j) {
      double2 a = zld<R>(A11 + i + (int64_t)j * n);
      if (i == j) a.y = 0.0;
      As[i + j * (NB + 1)] = a;
      As[j + i * (NB + 1)] = zconj(a);
      Ls[i + j * (NB + 1)] = zld<R>(L11 + i + (int64_t)j * n);
    }
  }
  if (lane < w) rds[lane] = ws_of(G, g).rd[c0 + lane];
  __syncwarp();
  const int c = lane;
  if (c < w) {                       // column c of X = L^-1 A, in place
    for (int i = 0; i < w; ++i) {
      double2 a0 = As[i + c * (NB + 1)], a1 = make_double2(0.0, 0.0);
      int k = 0;
      for (; k + 1 < i; k += 2) {
        a0 = zfms<R>(Ls[i + k * (NB + 1)], As[k + c * (NB + 1)], a0);
        a1 = zfms<R>(Ls[i + (k + 1) * (NB + 1)], As[k + 1 + c * (NB + 1)], a1);
      }
      if (k < i) a0 = zfms<R>(Ls[i + k * (NB + 1)], As[k + c * (NB + 1)], a0);
      As[i + c * (NB + 1)] = zscal<R>(zadd<R>(a0, a1), rds[i]);
    }
  }
  __syncwarp();
  double2 y[NB];
#pragma unroll
  for (int i = 0; i < NB; ++i) {     // column c of C = L^-1 X^H: right-hand side conj(X[c, :])
    if (i < w && c < w) {
      double2 a0 = zconj(As[c + i * (NB + 1)]), a1 = make_double2(0.0, 0.0);
#pragma unroll
      for (int k = 0; k < NB; ++k) {
        if (k < i) {
          if (k & 1) a1 = zfms<R>(Ls[i + k * (NB + 1)], y[k], a1);
          else a0 = zfms<R>(Ls[i + k * (NB + 1)], y[k], a0);
        }
      }
      y[i] = zscal<R>(zadd<R>(a0, a1), rds[i]);
    } else {
      y[i] = make_double2(0.0, 0.0);
    }
  }
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    if (c < w && i < w && i >= c) {
      double2 v = y[i];
      if (i == c) v.y = 0.0;
      zst<R>(A11 + i + (int64_t)c * n, v);
    }
  }
}

// A21 -= 1/2 L21 A11 for the m x NB panel below (c0, c0); A11 (reduced, Hermitian) staged whole.
template <bool R>
__global__ void __launch_bounds__(256) k_hemm_half(Grp G, int c0, int m) {
  const int g = blockIdx.y, p = G.prob[g];
  if (!live(G, p)) return;
  const int n = G.n;
  __shared__ double2 As[NB * (NB + 1)];
  double2* A11 = G.H + G.hs_off[p] + c0 + (int64_t)c0 * n;
  for (int e = threadIdx.x; e < NB * NB; e += 256) {
    const int i = e % NB, j = e / NB;
    if (i >= j) {
      double2 a = zld<R>(A11 + i + (int64_t)j * n);
      if (i == j) a.y = 0.0;
      As[i + j * (NB + 1)] = a;
      As[j + i * (NB + 1)] = zconj(a);
    }
  }
  __syncthreads();
  const int64_t e = (int64_t)blockIdx.x * 256 + threadIdx.x;
  if (e >= (int64_t)m * NB) return;
  const int r = (int)(e % m), j = (int)(e / m);
  const double2* L21 = G.S + G.hs_off[p] + (c0 + NB) + (int64_t)c0 * n;
  double2 s0 = make_double2(0.0, 0.0), s1 = s0;
#pragma unroll 8
  for (int k = 0; k < NB; k += 2) {
    s0 = zfma<R>(zld<R>(L21 + r + (int64_t)k * n), As[k + j * (NB + 1)], s0);
    s1 = zfma<R>(zld<R>(L21 + r + (int64_t)(k + 1) * n), As[k + 1 + j * (NB + 1)], s1);
  }
  double2* t = G.H + G.hs_off[p] + (c0 + NB + r) + (int64_t)(c0 + j) * n;
  const double2 s = zadd<R>(s0, s1);
  double2 a = zld<R>(t);
  a.x = fma(-0.5, s.x, a.x);
  if constexpr (!R) a.y = fma(-0.5, s.y, a.y);
  zst<R>(t, a);
}

// Deferred A21 <- L22^-1 A21 of every panel, chunk row t (rows t*NB ..): solve with the diagonal
// block of L for the t*NB columns left of it, one thread per column.
template <bool R>
__global__ void __launch_bounds__(128) k_trsm_diag(Grp G, int t) {
  const int g = blockIdx.y, p = G.prob[g];
  if (!live(G, p)) return;
  const int n = G.n, r0 = t * NB, h = min(NB, n - r0);
  __shared__ double2 Ls[NB * (NB + 1)];
  __shared__ double rds[NB];
  const double2* L = G.S + G.hs_off[p] + r0 + (int64_t)r0 * n;
  for (int e = threadIdx.x; e < h * h; e += 128) {
    const int i = e % h, j = e / h;
    if (i >= j) Ls[i + j * (NB + 1)] = zld<R>(L + i + (int64_t)j * n);
  }
  if (threadIdx.x < h) rds[threadIdx.x] = ws_of(G, g).rd[r0 + threadIdx.x];
  __syncthreads();
  const int c = blockIdx.x * 128 + threadIdx.x;
  if (c >= r0) return;
  double2* col = G.H + G.hs_off[p] + r0 + (int64_t)c * n;
  double2 x[NB];
#pragma unroll
  for (int i = 0; i < NB; ++i) {
    if (i < h) {
      double2 a0 = zld<R>(col + i), a1 = make_double2(0.0, 0.0);
#pragma unroll
      for (int k = 0; k < NB; ++k) {
        if (k < i) {
          if (k & 1) a1 = zfms<R>(Ls[i + k * (NB + 1)], x[k], a1);
          else a0 = zfms<R>(Ls[i + k * (NB + 1)], x[k], a0);
        }
      }
      x[i] = zscal<R>(zadd<R>(a0, a1), rds[i]);
      zst<R>(col + i, x[i]);
    } else {
      x[i] = make_double2(0.0, 0.0);
    }
  }
}

// Chunk row t's update of the rows below: H[r1:, 0:t*NB] -= L[r1:, t*NB : t*NB+NB] X, X the solved
// chunk H[t*NB : t*NB+NB, 0:t*NB], r1 = (t+1)*NB.  T x T output tiles ((T/4)^2 threads), ntj tile columns.
template <bool R, int T>
__global__ void __launch_bounds__((T / 4) * (T / 4)) k_gemm_nn(Grp G, int t, int ntj) {
  constexpr int NTH = (T / 4) * (T / 4);
  const int g = blockIdx.y, p = G.prob[g];
  if (!live(G, p)) return;
  const int n = G.n, r0 = t * NB, r1 = r0 + NB, mr = n - r1, nc = r0;
  const int I = blockIdx.x / ntj, J = blockIdx.x % ntj;
  extern __shared__ double2 smr[];
  double2* sP = smr;                 // [k][T rows]
  double2* sX = smr + KC * T;        // [k][T cols]
  const double2* Lp = G.S + G.hs_off[p] + r1 + (int64_t)r0 * n;   // rows r1.., columns r0..r0+NB
  const double2* Xp = G.H + G.hs_off[p] + r0;                      // rows r0..r0+NB, column c at Xp + c*n
  double2* C = G.H + G.hs_off[p] + r1;
  const int tid = threadIdx.x, tr = tid % (T / 4), tc = tid / (T / 4);
  double2 acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = make_double2(0.0, 0.0);
  for (int k0 = 0; k0 < NB; k0 += KC) {
    for (int e = tid; e < KC * T; e += NTH) {
      const int r = e % T, k = e / T;
      const int gi = I * T + r;
      sP[k * T + r] = gi < mr ? zld<R>(Lp + gi + (int64_t)(k0 + k) * n) : make_double2(0.0, 0.0);
      const int kx = e % KC, cx = e / KC;
      const int gc = J * T + cx;
      sX[kx * T + cx] = gc < nc ? zld<R>(Xp + (k0 + kx) + (int64_t)gc * n) : make_double2(0.0, 0.0);
    }
    __syncthreads();
#pragma unroll 2
    for (int k = 0; k < KC; ++k) {
      double2 a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) a[u] = sP[k * T + tr * 4 + u];
#pragma unroll
      for (int v = 0; v < 4; ++v) b[v] = sX[k * T + tc * 4 + v];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] = zfma<R>(a[u], b[v], acc[u][v]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const int c = J * T + tc * 4 + v;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int r = I * T + tr * 4 + u;
      if (r < mr && c < nc) {
        double2* q = C + r + (int64_t)c * n;
        zst<R>(q, zsub<R>(zld<R>(q), acc[u][v]));
      }
    }
  }
}

// ------------------------------------------------------------------ tridiagonalisation
// Panel at c0 (M = n - c0 rows and columns from there), column j of the panel.  V(r, q) is H at
// (c0 + r, c0 + q) for r > q (V(q+1, q) = 1 stored there during the panel); W(r, q) is W[q*n + c0 + r].

// 1. column j, rows j..M-1: a -= V(r, 0:j) W(j, 0:j)^H + W(r, 0:j) V(j, 0:j)^H; norm partial of
//    rows j+2.. (the reflector's x without its first entry).
template <bool R>
__global__ void __launch_bounds__(RC) k_tr_colupd(Grp G, int c0, int j) {
  const int g = blockIdx.y, p = G.prob[g];
  if (!live(G, p)) return;
  const int n = G.n, M = n - c0;
  const WS w = ws_of(G, g);
  double2* A = G.H + G.hs_off[p];
  __shared__ double2 vj[NB], wj[NB];
  __shared__ double red[RC / 32];
  if (threadIdx.x < j) {
    vj[threadIdx.x] = zld<R>(A + (c0 + j) + (int64_t)(c0 + threadIdx.x) * n);
    wj[threadIdx.x] = zld<R>(w.W + (int64_t)threadIdx.x * n + c0 + j);
  }
  __syncthreads();
  const int r = j + blockIdx.x * RC + threadIdx.x;
  double s2 = 0.0;
  if (r < M) {
    const int gr = c0 + r;
    double2* t = A + gr + (int64_t)(c0 + j) * n;
    double2 a = zld<R>(t);
    if (j > 0) {
      double2 a1 = make_double2(0.0, 0.0);
      for (int q = 0; q < j; ++q) {
        a = zfms_cj<R>(zld<R>(A + gr + (int64_t)(c0 + q) * n), wj[q], a);
        a1 = zfms_cj<R>(zld<R>(w.W + (int64_t)q * n + gr), vj[q], a1);
      }
      a = zadd<R>(a, a1);
      zst<R>(t, a);
    }
    if (r >= j + 2) s2 = R ? a.x * a.x : fma(a.x, a.x, a.y * a.y);
  }
  s2 = block_sum(s2, red);
  if (threadIdx.x == 0) w.r1[blockIdx.x] = make_double2(s2, 0.0);
}

// 2. the reflector of column j (one CTA per problem): beta, tau, v = x / (alpha - beta) with
//    v(0) = 1 stored in H and in w.v; d and e^2 of the tridiagonal.
template <bool R>
__global__ void __launch_bounds__(256) k_tr_reflect(Grp G, int c0, int j) {
  const int g = blockIdx.x, p = G.prob[g];
  if (!live(G, p)) return;
  const int n = G.n, M = n - c0, m = M - j - 1, k = c0 + j;
  const WS w = ws_of(G, g);
  double2* A = G.H + G.hs_off[p];
  double2* x = A + (k + 1) + (int64_t)k * n;
  __shared__ double2 s_scl;
  __shared__ int s_triv;
  double xnorm2 = 0.0;
  if (threadIdx.x < 32) xnorm2 = warp_chunk_sum<true>(w.r1, 1, cdiv_d(M - j, RC)).x;
  if (threadIdx.x == 0) {
    const double2 alpha = zld<R>(x);
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
      const double dr = alpha.x - beta, di = alpha.y;
      const double den = 1.0 / fma(dr, dr, di * di);
      scl = make_double2(dr * den, -di * den);
    }
    w.sc[0] = make_double2(taur, R ? 0.0 : taui);
    w.sc[1] = scl;
    w.sc[2] = make_double2((double)trivial, 0.0);
    w.d[k] = A[k + (int64_t)k * n].x;
    w.e2[k] = beta * beta;
    zst<R>(x, make_double2(1.0, 0.0));
    zst<R>(w.v, make_double2(1.0, 0.0));
    s_scl = scl;
    s_triv = trivial;
  }
  __syncthreads();
  const double2 scl = s_scl;
  const int trivial = s_triv;
  for (int i = 1 + threadIdx.x; i < m; i += 256) {
    double2 v = zld<R>(x + i);
    if (!trivial) {
      v = zmul<R>(v, scl);
      zst<R>(x + i, v);
    }
    zst<R>(w.v + i, v);
  }
}

// 3. y = A22 v, A22 the m x m trailing matrix at (base, base) as it stood at the panel's start.
//    One CTA per 64x64 tile (I, J) of its lower triangle, read once for both products: A_IJ v_J goes
//    to partial slot J of the rows of block I, A_IJ^H v_I to slot I of the rows of block J; a
//    diagonal tile gives its whole Hermitian block product to slot I.  Every (block, slot) pair is
//    written once per column.
template <bool R>
__global__ void __launch_bounds__(256) k_tr_hemv(Grp G, int base, int m) {
  const int g = blockIdx.y, p = G.prob[g];
  if (!live(G, p)) return;
  const WS w = ws_of(G, g);
  if (w.sc[2].x != 0.0) return;                  // trivial reflector: w = 0
  const int n = G.n;
  int I, J;
  tile_ij(blockIdx.x, I, J);
  extern __shared__ double2 smr[];
  double2* T = smr;                              // [TS][TLD], column-major
  double2* vI = smr + TS * TLD;
  double2* vJ = vI + TS;
  const double2* A22 = G.H + G.hs_off[p] + base + (int64_t)base * n;
  const int tid = threadIdx.x;
  for (int e = tid; e < TS * TS; e += 256) {
    const int r = e & (TS - 1), c = e >> 6;
    const int gi = I * TS + r, gj = J * TS + c;
    double2 a = make_double2(0.0, 0.0);
    if (gi < m && gj < m && (I > J || r >= c)) {
      a = zld<R>(A22 + gi + (int64_t)gj * n);
      if (gi == gj) a.y = 0.0;
    }
    T[r + c * TLD] = a;
  }
  if (tid < TS) {
    const int gi = I * TS + tid;
    vI[tid] = gi < m ? zld<R>(w.v + gi) : make_double2(0.0, 0.0);
  } else if (tid < 2 * TS) {
    const int gj = J * TS + tid - TS;
    vJ[tid - TS] = gj < m ? zld<R>(w.v + gj) : make_double2(0.0, 0.0);
  }
  __syncthreads();
  const int r = tid & (TS - 1), q = tid >> 6;
  double2 dir0 = make_double2(0.0, 0.0), dir1 = dir0, tr0 = dir0, tr1 = dir0;
#pragma unroll
  for (int c = 0; c < 16; c += 2) {
    dir0 = zfma<R>(T[r + (q * 16 + c) * TLD], vJ[q * 16 + c], dir0);
    dir1 = zfma<R>(T[r + (q * 16 + c + 1) * TLD], vJ[q * 16 + c + 1], dir1);
  }
  const double2* Tc = T + r * TLD;               // column r
#pragma unroll
  for (int c = 0; c < 16; c += 2) {
    const int r0 = q * 16 + c, r1 = r0 + 1;
    if (I != J || r0 != r) tr0 = zfma_cja<R>(Tc[r0], vI[r0], tr0);
    if (I != J || r1 != r) tr1 = zfma_cja<R>(Tc[r1], vI[r1], tr1);
  }
  __syncthreads();                               // the tile is no longer read: reuse it for partials
  double2* pd = smr;                             // [4][TS]
  double2* pt = smr + 4 * TS;
  pd[q * TS + r] = zadd<R>(dir0, dir1);
  pt[q * TS + r] = zadd<R>(tr0, tr1);
  __syncthreads();
  if (tid < TS) {
    double2 yd = pd[tid], yt = pt[tid];
#pragma unroll
    for (int qq = 1; qq < 4; ++qq) {
      yd = zadd<R>(yd, pd[qq * TS + tid]);
      yt = zadd<R>(yt, pt[qq * TS + tid]);
    }
    const int gi = I * TS + tid, gj = J * TS + tid;
    if (I == J) {
      if (gi < m) zst<R>(w.Yp + (int64_t)I * n + gi, zadd<R>(yd, yt));
    } else {
      if (gi < m) zst<R>(w.Yp + (int64_t)J * n + gi, yd);
      if (gj < m) zst<R>(w.Yp + (int64_t)I * n + gj, yt);
    }
  }
}

// 4. y = sum of the hemv slots (fixed order) for this chunk's rows; partial dot products
//    W(:, q)^H v and V(:, q)^H v over the chunk for the panel's earlier columns q < j (warp per
//    product, lanes over rows, fixed reduction tree).
template <bool R>
__global__ void __launch_bounds__(256) k_tr_dots(Grp G, int c0, int j) {
  const int g = blockIdx.y, p = G.prob[g];
  if (!live(G, p)) return;
  const WS w = ws_of(G, g);
  if (w.sc[2].x != 0.0) return;
  const int n = G.n, m = n - c0 - j - 1, nt = cdiv_d(m, TS);
  const double2* A = G.H + G.hs_off[p];
  __shared__ double2 vloc[RC];
  if (threadIdx.x < RC) {
    const int i = blockIdx.x * RC + threadIdx.x;
    if (i < m) {
      double2 y = zld<R>(w.Yp + i);
      for (int s = 1; s < nt; ++s) y = zadd<R>(y, zld<R>(w.Yp + (int64_t)s * n + i));
      zst<R>(w.y + i, y);
      vloc[threadIdx.x] = zld<R>(w.v + i);
    } else {
      vloc[threadIdx.x] = make_double2(0.0, 0.0);
    }
  }
  if (j == 0) return;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row0 = c0 + j + 1 + blockIdx.x * RC;     // global row of the chunk's first row
  for (int dq = warp; dq < 2 * j; dq += 8) {
    const double2* src = dq < j ? w.W + (int64_t)dq * n : A + (int64_t)(c0 + dq - j) * n;
    double2 acc = make_double2(0.0, 0.0);
#pragma unroll
    for (int rr = lane; rr < RC; rr += 32) {
      if (blockIdx.x * RC + rr < m) acc = zfma_cja<R>(zld<R>(src + row0 + rr), vloc[rr], acc);
    }
    for (int o = 16; o > 0; o >>= 1) {
      acc.x += __shfl_xor_sync(0xffffffffu, acc.x, o);
      if constexpr (!R) acc.y += __shfl_xor_sync(0xffffffffu, acc.y, o);
    }
    if (lane == 0) zst<R>(w.r2 + (int64_t)blockIdx.x * 2 * NB + dq, acc);
  }
}

// 5. y -= V (W^H v) + W (V^H v); w = tau y stored as W(:, j); partial w^H v.
template <bool R>
__global__ void __launch_bounds__(RC) k_tr_wupd(Grp G, int c0, int j) {
  const int g = blockIdx.y, p = G.prob[g];
  if (!live(G, p)) return;
  const WS w = ws_of(G, g);
  const int n = G.n, m = n - c0 - j - 1, nch = cdiv_d(m, RC);
  const int i = blockIdx.x * RC + threadIdx.x;
  const int gr = c0 + j + 1 + i;
  __shared__ double red[2 * (RC / 32)];
  if (w.sc[2].x != 0.0) {                         // trivial reflector: W(:, j) = 0
    if (i < m) zst<R>(w.W + (int64_t)j * n + gr, make_double2(0.0, 0.0));
    if (threadIdx.x == 0) w.r3[blockIdx.x] = make_double2(0.0, 0.0);
    return;
  }
  const double2* A = G.H + G.hs_off[p];
  __shared__ double2 t12[2 * NB];
  for (int dq = threadIdx.x >> 5; dq < 2 * j; dq += RC / 32) {   // [0, j): W^H v, [j, 2j): V^H v
    const double2 sdq = warp_chunk_sum<R>(w.r2 + dq, 2 * NB, nch);
    if ((threadIdx.x & 31) == 0) t12[dq] = sdq;
  }
  __syncthreads();
  const double2 tau = w.sc[0];
  double pr = 0.0, pi = 0.0;
  if (i < m) {
    double2 y0 = zld<R>(w.y + i), y1 = make_double2(0.0, 0.0), y2 = y1, y3 = y1;
    int q = 0;
    for (; q + 1 < j; q += 2) {        // two columns per step: four independent chains, four loads ahead
      const double2 v0 = zld<R>(A + gr + (int64_t)(c0 + q) * n), v1 = zld<R>(A + gr + (int64_t)(c0 + q + 1) * n);
      const double2 w0 = zld<R>(w.W + (int64_t)q * n + gr), w1 = zld<R>(w.W + (int64_t)(q + 1) * n + gr);
      y0 = zfms<R>(v0, t12[q], y0);
      y1 = zfms<R>(w0, t12[j + q], y1);
      y2 = zfms<R>(v1, t12[q + 1], y2);
      y3 = zfms<R>(w1, t12[j + q + 1], y3);
    }
    if (q < j) {
      y0 = zfms<R>(zld<R>(A + gr + (int64_t)(c0 + q) * n), t12[q], y0);
      y1 = zfms<R>(zld<R>(w.W + (int64_t)q * n + gr), t12[j + q], y1);
    }
    const double2 wi = zmul<R>(tau, zadd<R>(zadd<R>(y0, y2), zadd<R>(y1, y3)));
    zst<R>(w.W + (int64_t)j * n + gr, wi);
    const double2 vi = zld<R>(w.v + i);
    if constexpr (R) {
      pr = wi.x * vi.x;
    } else {
      pr = fma(wi.x, vi.x, wi.y * vi.y);
      pi = fma(wi.x, vi.y, -wi.y * vi.x);
    }
  }
  pr = block_sum(pr, red);
  if constexpr (!R) pi = block_sum(pi, red + RC / 32);
  if (threadIdx.x == 0) w.r3[blockIdx.x] = make_double2(pr, pi);
}

// 6. W(:, j) += (-tau/2 w^H v) v.
template <bool R>
__global__ void __launch_bounds__(RC) k_tr_wfin(Grp G, int c0, int j) {
  const int g = blockIdx.y, p = G.prob[g];
  if (!live(G, p)) return;
  const WS w = ws_of(G, g);
  if (w.sc[2].x != 0.0) return;
  const int n = G.n, m = n - c0 - j - 1, nch = cdiv_d(m, RC);
  __shared__ double2 s_al;
  if (threadIdx.x < 32) {
    const double2 s = warp_chunk_sum<R>(w.r3, 1, nch);
    const double2 tau = w.sc[0];
    if (threadIdx.x == 0) s_al = zmul<R>(make_double2(-0.5 * tau.x, -0.5 * tau.y), s);
  }
  __syncthreads();
  const int i = blockIdx.x * RC + threadIdx.x;
  if (i >= m) return;
  double2* t = w.W + (int64_t)j * n + (c0 + j + 1 + i);
  zst<R>(t, zfma<R>(s_al, zld<R>(w.v + i), zld<R>(t)));
}

// ------------------------------------------------------------------ eigenvalues
// Last diagonal entry, Gershgorin bounds, FP32 copies of the tridiagonal (one CTA per problem).
template <bool R>
__global__ void __launch_bounds__(256) k_tri_bounds(Grp G) {
  const int g = blockIdx.x, p = G.prob[g];
  if (!live(G, p)) return;
  const int n = G.n, tid = threadIdx.x;
  const WS w = ws_of(G, g);
  __shared__ double red[3 * 8];
  if (tid == 0) w.d[n - 1] = (G.H + G.hs_off[p])[(int64_t)(n - 1) * (n + 1)].x;
  __syncthreads();
  double lo = 1e300, hi = -1e300, emax = 0.0;
  for (int i = tid; i < n; i += 256) {
    const double ea = (i > 0) ? sqrt(w.e2[i - 1]) : 0.0;
    const double eb = (i < n - 1) ? sqrt(w.e2[i]) : 0.0;
    lo = fmin(lo, w.d[i] - ea - eb);
    hi = fmax(hi, w.d[i] + ea + eb);
    if (i < n - 1) emax = fmax(emax, w.e2[i]);
    w.d32[i] = (float)w.d[i];
    w.e232[i] = (i < n - 1) ? (float)w.e2[i] : 0.0f;
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    emax = fmax(emax, __shfl_xor_sync(0xffffffffu, emax, o));
  }
  if ((tid & 31) == 0) {
    red[tid >> 5] = lo;
    red[8 + (tid >> 5)] = hi;
    red[16 + (tid >> 5)] = emax;
  }
  __syncthreads();
  if (tid == 0) {
    for (int q = 1; q < 8; ++q) {
      red[0] = fmin(red[0], red[q]);
      red[8] = fmax(red[8], red[8 + q]);
      red[16] = fmax(red[16], red[16 + q]);
    }
    w.sc[3] = make_double2(red[0], red[8]);
    w.sc[4] = make_double2(red[16], 0.0);
  }
}

__global__ void __launch_bounds__(128) k_tri_eig(Grp G) {
  const int g = blockIdx.y, p = G.prob[g];
  const int n = G.n, j = blockIdx.x * 128 + threadIdx.x;
  if (j >= n) return;
  const int st = G.status[p];
  double* out = G.eig + G.eig_off[p];
  if (st == SKN_ERR_NOT_SPD) {
    out[j] = __longlong_as_double(0x7ff8000000000000LL);
    return;
  }
  if (st != SKN_OK) return;
  const WS w = ws_of(G, g);
  const double2 lh = w.sc[3];
  const skn_sturm::Bounds B = skn_sturm::make_bounds(lh.x, lh.y, w.sc[4].x, n);
  out[j] = skn_sturm::eigenvalue(w.d, w.e2, w.d32, w.e232, n, j, B);
}

// ------------------------------------------------------------------ host sequence
constexpr int SM_HEMV = (TS * TLD + 2 * TS) * (int)sizeof(double2);    // 67 KB
static_assert(8 * TS <= TS * TLD, "hemv partials fit in the tile's space");
constexpr int sm_r2k(int mode, int t) { return (mode ? 4 : 2) * KC * t * (int)sizeof(double2); }   // <= 64 KB
constexpr int sm_gemm(int t) { return 2 * KC * t * (int)sizeof(double2); }

// Dynamic shared memory of k_r2k_tc: the B slices and two stages of A slices (real: 60 KB, complex: 184 KB),
// the real variant padded to 96 KB so that at most two CTAs share an SM, as many as its 256 TMEM columns each
// allow.
constexpr int tc_smem(bool real) { return real ? 96 * 1024 : TCS * 32 * 128 * 2 + 2 * 2 * 128 * 128 * 2; }
static_assert(TCS * 32 * 64 * 2 + 2 * 128 * 64 * 2 <= 96 * 1024, "real slices fit the padded region");
static_assert(TCS * 32 * 128 * 2 + 2 * 2 * 128 * 128 * 2 <= 227 * 1024, "complex slices fit shared memory");
constexpr int TC_MIN_M = 512;    // trailing matrices from this size up take the tensor-core update when asked

template <bool R>
cudaError_t set_attrs() {
  cudaError_t e = cudaFuncSetAttribute(k_rank2k<R, 1, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm_r2k(1, 64));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_tr_hemv<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, SM_HEMV);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_r2k_tc<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, tc_smem(R));
  return e;
}

inline unsigned tri_tiles(int m, int t = TS) {
  const int nt = cdiv(m, t);
  return (unsigned)(nt * (nt + 1) / 2);
}

// Tile edge for a product kernel: 64 unless its grid would fill fewer than two waves of the GPU's SMs.
inline bool small_tiles(int64_t tiles64, int n_prob, int sms) { return tiles64 * n_prob < 2LL * sms; }

template <bool R, int MODE>
void rank2k(const Grp& G, Mat C, int m, Mat P, Mat Q, int K, int sms, bool tc, cudaStream_t st) {
  const unsigned Pn = (unsigned)G.n_prob;
  if (tc && m >= TC_MIN_M) {          // slices of the panel's rows, then the tensor-core tiles
    k_r2k_split<R, MODE><<<dim3(cdiv(m, 8), Pn), 256, 0, st>>>(G, P, Q, m, K);
    k_r2k_tc<R><<<dim3((unsigned)(cdiv(m, 128) * cdiv(m, 32)), Pn), 128, tc_smem(R), st>>>(G, C, m);
    return;
  }
  if (small_tiles(tri_tiles(m, 64), G.n_prob, sms))
    k_rank2k<R, MODE, 32><<<dim3(tri_tiles(m, 32), Pn), 64, sm_r2k(MODE, 32), st>>>(G, C, m, P, Q, K);
  else
    k_rank2k<R, MODE, 64><<<dim3(tri_tiles(m, 64), Pn), 256, sm_r2k(MODE, 64), st>>>(G, C, m, P, Q, K);
}

template <bool R>
void gemm_nn(const Grp& G, int t, int sms, cudaStream_t st) {
  const int n = G.n;
  const unsigned Pn = (unsigned)G.n_prob;
  const int64_t t64 = (int64_t)cdiv(n - (t + 1) * NB, 64) * cdiv(t * NB, 64);
  if (small_tiles(t64, G.n_prob, sms)) {
    const int ntj = cdiv(t * NB, 32);
    k_gemm_nn<R, 32><<<dim3((unsigned)(cdiv(n - (t + 1) * NB, 32) * ntj), Pn), 64, sm_gemm(32), st>>>(G, t, ntj);
  } else {
    const int ntj = cdiv(t * NB, 64);
    k_gemm_nn<R, 64><<<dim3((unsigned)(cdiv(n - (t + 1) * NB, 64) * ntj), Pn), 256, sm_gemm(64), st>>>(G, t, ntj);
  }
}

template <bool R>
void run(const Grp& G, bool tc, cudaStream_t st) {
  const int n = G.n;
  const unsigned P = (unsigned)G.n_prob;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms < 1) sms = 1;
  k_init<<<dim3(cdiv(2 * n, 256), P), 256, 0, st>>>(G);
  k_zscan<R><<<dim3(cdiv(n, 256), cdiv(n, 256), 2 * P), 256, 0, st>>>(G);
  k_zfix<R><<<dim3(cdiv(n, 256), 2 * P), 256, 0, st>>>(G);
  // Cholesky of S
  for (int c0 = 0; c0 < n; c0 += NB) {
    const int w = min(NB, n - c0), m = n - c0 - w;
    k_potrf<R><<<P, 32, 0, st>>>(G, c0, w);
    if (m > 0) {
      k_trsm_right<R><<<dim3(cdiv(m, RC), P), RC, 0, st>>>(G, 1, c0, m);
      rank2k<R, 0>(G, Mat{1, (int64_t)(c0 + NB) * (n + 1)}, m, Mat{1, (c0 + NB) + (int64_t)c0 * n}, Mat{1, 0}, NB,
                   sms, tc, st);
    }
  }
  // reduction to standard form, the panels' left solves deferred
  for (int c0 = 0; c0 < n; c0 += NB) {
    const int w = min(NB, n - c0), m = n - c0 - w;
    k_hegs2<R><<<P, 32, 0, st>>>(G, c0, w);
    if (m > 0) {
      k_trsm_right<R><<<dim3(cdiv(m, RC), P), RC, 0, st>>>(G, 0, c0, m);
      k_hemm_half<R><<<dim3(cdiv(m * NB, 256), P), 256, 0, st>>>(G, c0, m);
      rank2k<R, 1>(G, Mat{0, (int64_t)(c0 + NB) * (n + 1)}, m, Mat{0, (c0 + NB) + (int64_t)c0 * n},
                   Mat{1, (c0 + NB) + (int64_t)c0 * n}, NB, sms, tc, st);
      k_hemm_half<R><<<dim3(cdiv(m * NB, 256), P), 256, 0, st>>>(G, c0, m);
    }
  }
  const int T = cdiv(n, NB);
  for (int t = 1; t < T; ++t) {
    k_trsm_diag<R><<<dim3(cdiv(t * NB, 128), P), 128, 0, st>>>(G, t);
    if ((t + 1) * NB < n) gemm_nn<R>(G, t, sms, st);
  }
  // tridiagonalisation
  for (int c0 = 0; c0 < n - 1; c0 += NB) {
    const int w = min(NB, n - 1 - c0), M = n - c0;
    for (int j = 0; j < w; ++j) {
      const int m = M - j - 1;
      k_tr_colupd<R><<<dim3(cdiv(M - j, RC), P), RC, 0, st>>>(G, c0, j);
      k_tr_reflect<R><<<P, 256, 0, st>>>(G, c0, j);
      k_tr_hemv<R><<<dim3(tri_tiles(m), P), 256, SM_HEMV, st>>>(G, c0 + j + 1, m);
      k_tr_dots<R><<<dim3(cdiv(m, RC), P), 256, 0, st>>>(G, c0, j);
      k_tr_wupd<R><<<dim3(cdiv(m, RC), P), RC, 0, st>>>(G, c0, j);
      k_tr_wfin<R><<<dim3(cdiv(m, RC), P), RC, 0, st>>>(G, c0, j);
    }
    const int m2 = M - w;
    if (m2 > 0)
      rank2k<R, 1>(G, Mat{0, (int64_t)(c0 + w) * (n + 1)}, m2, Mat{0, (c0 + w) + (int64_t)c0 * n}, Mat{2, c0 + w}, w,
                   sms, tc, st);
  }
  k_tri_bounds<R><<<P, 256, 0, st>>>(G);
  k_tri_eig<<<dim3(cdiv(n, 128), P), 128, 0, st>>>(G);
}

}  // namespace

extern "C" int skn_eigh_wide_scratch_bytes(int n_prob, int n, int64_t* bytes) {
  if (!bytes || n_prob < 0 || n < 1) return SKN_ERR_ARG;
  if (n > WIDE_MAX_N) return SKN_ERR_CAPACITY;
  *bytes = (int64_t)n_prob * layout(n).stride * (int64_t)sizeof(double2);
  return SKN_OK;
}

static int wide_entry(int n_prob, int n, const int32_t* prob, const int32_t* nvec, const int64_t* hs_off,
                      const int64_t* eig_off, double* H, double* S, double* eig, int32_t* status, double* scratch,
                      int64_t scratch_bytes, int real, bool tc, cudaStream_t stream) {
  if (n_prob < 0 || n < 1) return SKN_ERR_ARG;
  if (n_prob == 0) return SKN_OK;
  if (n_prob > 32767) return SKN_ERR_CAPACITY;   // grid z of the zero-row scan holds 2 n_prob
  if (!prob || !nvec || !hs_off || !eig_off || !H || !S || !eig || !status || !scratch) return SKN_ERR_ARG;
  if (n > WIDE_MAX_N) return SKN_ERR_CAPACITY;
  if (scratch_bytes < (int64_t)n_prob * layout(n).stride * (int64_t)sizeof(double2)) return SKN_ERR_CAPACITY;
  if ((reinterpret_cast<uintptr_t>(scratch) & 15) != 0 || (reinterpret_cast<uintptr_t>(H) & 15) != 0 ||
      (reinterpret_cast<uintptr_t>(S) & 15) != 0)
    return SKN_ERR_ARG;
  if ((real ? set_attrs<true>() : set_attrs<false>()) != cudaSuccess) return SKN_ERR_CUDA;
  Grp G{n, n_prob, prob, nvec, hs_off, eig_off, (double2*)H, (double2*)S, eig, status, (double2*)scratch};
  if (real)
    run<true>(G, tc, stream);
  else
    run<false>(G, tc, stream);
  return cudaPeekAtLastError() == cudaSuccess ? SKN_OK : SKN_ERR_CUDA;
}


extern "C" int skn_eigh_gen_wide(int n_prob, int n, const int32_t* prob, const int32_t* nvec, const int64_t* hs_off,
                                 const int64_t* eig_off, double* H, double* S, double* eig, int32_t* status,
                                 double* scratch, int64_t scratch_bytes, int real, cudaStream_t stream) {
  return wide_entry(n_prob, n, prob, nvec, hs_off, eig_off, H, S, eig, status, scratch, scratch_bytes, real, false,
                    stream);
}

extern "C" int skn_eigh_gen_wide_tc(int n_prob, int n, const int32_t* prob, const int32_t* nvec,
                                    const int64_t* hs_off, const int64_t* eig_off, double* H, double* S, double* eig,
                                    int32_t* status, double* scratch, int64_t scratch_bytes, int real,
                                    cudaStream_t stream) {
  return wide_entry(n_prob, n, prob, nvec, hs_off, eig_off, H, S, eig, status, scratch, scratch_bytes, real, true,
                    stream);
}
