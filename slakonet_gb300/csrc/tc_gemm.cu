// FP64-accurate GEMM on the bf16 tensor cores (tcgen05), by error-free splitting.
//
// GB300 runs FP64 at ~1.25 TFLOP/s, and its FP64 tensor instruction (DMMA) at
// the same rate, so the only tensor-core route for the eigensolver's
// GEMM-shaped FP64 updates is emulation.  The scheme here is the splitting of
// Ozaki, Ogita and Oishi ("Error-free transformations of matrix multiplication
// by using fast routines of matrix multiplication and its applications",
// Numer. Algorithms 59, 2012) with integer slices:
//   A[i,:] = 2^ea_i * sum_s a_s[i,:] 2^(-8(s+1)),  a_s integers, |a_s| <= 256,
//   B[j,:] = 2^eb_j * sum_t b_t[j,:] 2^(-8(t+1)),
// every slice held exactly in bf16 (8 significant bits).  A product of two
// slices is an integer below 2^16 and exact in FP32; a sum of at most 256 of
// them stays within 2^24, so a K chunk of 256 accumulates exactly in the
// tensor core's FP32 accumulator -- provided the accumulator really is exact
// for such sums, which tests/test_gpu_tc_gemm.py measures on the GPU.  The
// slice products with s + t < S are scaled by powers of two and summed in
// FP64; with S = 7 slices (56 bits) the dropped terms lie below FP64 rounding.
//
// k_tc_gemm: one CTA (4 warps) per 128 x 128 output tile, D = A B^T with A
// [M x K] and B [N x K] bf16, K contiguous.  K advances in 64-wide stages:
// the warps copy the two 128 x 64 tiles into shared memory in the
// no-swizzle K-major core-matrix layout (8 rows x 16 bytes per core matrix),
// one thread issues four tcgen05.mma (M 128, N 128, K 16) accumulating in
// 128 TMEM columns, and tcgen05.commit signals an mbarrier the warps wait on
// (with an iteration limit) before the next stage overwrites the tiles.  The
// epilogue reads the accumulator with tcgen05.ld (each warp its 32 TMEM
// lanes) and either stores FP32 or adds the scaled values into an FP64 C.
#include <cuda_bf16.h>

#include "skn_common.cuh"

namespace {

constexpr int TM = 128, TN = 128, TK = 64;         // CTA tile and K stage
constexpr int TC_THREADS = 128;
constexpr uint32_t LBO = 128;                      // bytes between core matrices along K
constexpr uint32_t SBO = (TK / 8) * 128;           // bytes between core matrices along M/N
constexpr int TILE_BYTES = TM * TK * 2;            // one 128 x 64 bf16 tile
constexpr uint32_t TMEM_COLS = 128;
constexpr long long WAIT_LIMIT = 1LL << 26;        // mbarrier polls before giving up

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: no swizzle, K-major core matrices.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)((LBO >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((SBO >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;                          // descriptor version for tcgen05
  return d;                                        // base offset 0, layout type 0 (no swizzle)
}

// Instruction descriptor, kind::f16: D F32, A and B BF16, both K-major, M = 128, N = 128.
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(TN >> 3) << 17) |
                           ((uint32_t)(TM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t"
      "}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(IDESC), "r"(accumulate));
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (long long it = 0; it < WAIT_LIMIT; ++it) {
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

// Copy rows [r0, r0 + 128) x K-columns [k0, k0 + 64) of a row-major bf16 matrix (ld elements) into the
// core-matrix layout: row r, 8-element group g at (r / 8) * SBO + g * LBO + (r % 8) * 16.
__device__ __forceinline__ void stage_tile(uint8_t* dst, const uint16_t* __restrict__ src, int64_t ld, int r0, int k0) {
  for (int v = threadIdx.x; v < TM * (TK / 8); v += TC_THREADS) {
    const int r = v / (TK / 8), g = v % (TK / 8);
    const uint4 x = *reinterpret_cast<const uint4*>(src + (int64_t)(r0 + r) * ld + k0 + g * 8);
    *reinterpret_cast<uint4*>(dst + (r / 8) * SBO + g * LBO + (r % 8) * 16) = x;
  }
}

// EPI 0: D[M x N] (FP32, row-major) = A B^T.
// EPI 1: C[i, j] += 2^(ea[i] + eb[j] + shift) * (A B^T)[i, j] in FP64 (row-major, ldc).
template <int EPI>
__global__ void __launch_bounds__(TC_THREADS) k_tc_gemm(const uint16_t* __restrict__ A, const uint16_t* __restrict__ B,
                                                        int K, int64_t lda, int64_t ldb, float* __restrict__ D,
                                                        int64_t ldd, double* __restrict__ C, int64_t ldc,
                                                        const int32_t* __restrict__ ea, const int32_t* __restrict__ eb,
                                                        int shift, int32_t* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sa = smem;
  uint8_t* sb = smem + TILE_BYTES;
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_slot;
  __shared__ int s_fail;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * TM, n0 = blockIdx.y * TN;
  const uint32_t bar_a = smem_u32(&bar);
  if (threadIdx.x == 0) {
    s_fail = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_a));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_slot;
  uint32_t phase = 0;
  for (int k0 = 0; k0 < K; k0 += TK) {
    stage_tile(sa, A, lda, m0, k0);
    stage_tile(sb, B, ldb, n0, k0);
    asm volatile("fence.proxy.async.shared::cta;");   // the tiles are read by the tensor core (async proxy)
    __syncthreads();
    if (threadIdx.x == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
#pragma unroll
      for (int kk = 0; kk < TK / 16; ++kk)
        mma_bf16(tmem, sdesc(a0 + kk * 2 * LBO), sdesc(b0 + kk * 2 * LBO), (k0 > 0 || kk > 0) ? 1u : 0u);
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar_a));
    }
    if (!mbar_wait(bar_a, phase)) s_fail = 1;
    phase ^= 1u;
    __syncthreads();
    if (s_fail) break;
  }
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (!s_fail) {
    // warp w holds TMEM lanes 32w .. 32w + 31 = output rows m0 + 32w + lane
    const int row = m0 + warp * 32 + lane;
    for (int c0 = 0; c0 < TN; c0 += 32) {
      uint32_t v[32];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
          "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
            "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]),
            "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]),
            "=r"(v[30]), "=r"(v[31])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;");
      if (EPI == 0) {
        float* d = D + (int64_t)row * ldd + n0 + c0;
#pragma unroll
        for (int q = 0; q < 32; q += 4)
          *reinterpret_cast<float4*>(d + q) = make_float4(__uint_as_float(v[q]), __uint_as_float(v[q + 1]),
                                                          __uint_as_float(v[q + 2]), __uint_as_float(v[q + 3]));
      } else {
        double* c = C + (int64_t)row * ldc + n0 + c0;
        const int er = ea[row] + shift;
#pragma unroll
        for (int q = 0; q < 32; ++q) c[q] += ldexp((double)__uint_as_float(v[q]), er + eb[n0 + c0 + q]);
      }
    }
  } else if (threadIdx.x == 0) {
    atomicExch(err, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
}

// Row split of an FP64 matrix X [R x K] (row-major, ld) into S bf16 integer slices
// (slices [S][R][K], K contiguous) and the row exponent e[r] with max |X[r,:]| < 2^e[r].
// One warp per row.
__global__ void k_split_rows(const double* __restrict__ X, int R, int K, int64_t ld, int S,
                             uint16_t* __restrict__ slices, int32_t* __restrict__ e) {
  const int lane = threadIdx.x & 31;
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (r >= R) return;
  const double* x = X + (int64_t)r * ld;
  double amax = 0.0;
  for (int k = lane; k < K; k += 32) amax = fmax(amax, fabs(x[k]));
  for (int o = 16; o > 0; o >>= 1) amax = fmax(amax, __shfl_xor_sync(0xffffffffu, amax, o));
  int ex = 0;
  if (amax > 0.0) frexp(amax, &ex);                // amax = f 2^ex, f in [0.5, 1)
  if (lane == 0) e[r] = ex;
  for (int k = lane; k < K; k += 32) {
    double v = ldexp(x[k], -ex);                   // |v| < 1, exact
    for (int s = 0; s < S; ++s) {
      v *= 256.0;                                  // exact (power of two)
      const double d = rint(v);                    // |d| <= 256
      v -= d;                                      // exact: the remainder of a rounding to integer
      slices[((int64_t)s * R + r) * K + k] = __bfloat16_as_ushort(__double2bfloat16(d));   // exact: |d| <= 256
    }
  }
}

cudaError_t set_tc_smem() {
  cudaError_t e = cudaFuncSetAttribute(k_tc_gemm<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * TILE_BYTES);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_tc_gemm<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * TILE_BYTES);
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace

extern "C" int skn_tc_gemm_bf16(const uint16_t* A, const uint16_t* B, float* D, int M, int N, int K, int32_t* err,
                                cudaStream_t stream) {
  if (M < 0 || N < 0 || K < 0) return SKN_ERR_ARG;
  if (M == 0 || N == 0) return SKN_OK;
  if (!A || !B || !D || !err) return SKN_ERR_ARG;
  if (M % TM || N % TN || K % TK || K == 0) return SKN_ERR_ARG;
  if (!aligned16(A) || !aligned16(B) || !aligned16(D)) return SKN_ERR_ARG;
  if (set_tc_smem() != cudaSuccess) return SKN_ERR_CUDA;
  k_tc_gemm<0><<<dim3(M / TM, N / TN), TC_THREADS, 2 * TILE_BYTES, stream>>>(A, B, K, K, K, D, N, nullptr, 0, nullptr,
                                                                             nullptr, 0, err);
  return cudaPeekAtLastError() == cudaSuccess ? SKN_OK : SKN_ERR_CUDA;
}

extern "C" int skn_gemm_f64_emulated_scratch_bytes(int M, int N, int K, int slices, int64_t* bytes) {
  if (!bytes || M < 0 || N < 0 || K < 0 || slices < 1 || slices > 8) return SKN_ERR_ARG;
  const int64_t sl = (int64_t)slices * ((int64_t)M + N) * K * 2;
  *bytes = ((sl + 255) / 256) * 256 + 4 * ((int64_t)M + N);
  return SKN_OK;
}

extern "C" int skn_gemm_f64_emulated(const double* A, const double* B, double* C, int M, int N, int K, int slices,
                                     void* scratch, int64_t scratch_bytes, int32_t* err, cudaStream_t stream) {
  if (M < 0 || N < 0 || K < 0 || slices < 1 || slices > 8) return SKN_ERR_ARG;
  if (M == 0 || N == 0) return SKN_OK;
  if (!A || !B || !C || !scratch || !err) return SKN_ERR_ARG;
  if (M % TM || N % TN || K % 256 || K == 0) return SKN_ERR_ARG;
  if (!aligned16(A) || !aligned16(B) || !aligned16(C) || !aligned16(scratch)) return SKN_ERR_ARG;
  int64_t need = 0;
  skn_gemm_f64_emulated_scratch_bytes(M, N, K, slices, &need);
  if (scratch_bytes < need) return SKN_ERR_CAPACITY;
  uint16_t* sa = static_cast<uint16_t*>(scratch);
  uint16_t* sb = sa + (int64_t)slices * M * K;
  const int64_t sl = (int64_t)slices * ((int64_t)M + N) * K * 2;
  int32_t* ea = reinterpret_cast<int32_t*>(static_cast<uint8_t*>(scratch) + ((sl + 255) / 256) * 256);
  int32_t* eb = ea + M;
  if (set_tc_smem() != cudaSuccess) return SKN_ERR_CUDA;
  if (cudaMemsetAsync(C, 0, sizeof(double) * (size_t)M * N, stream) != cudaSuccess) return SKN_ERR_CUDA;
  k_split_rows<<<(M + 7) / 8, 256, 0, stream>>>(A, M, K, K, slices, sa, ea);
  k_split_rows<<<(N + 7) / 8, 256, 0, stream>>>(B, N, K, K, slices, sb, eb);
  // slice pairs s + t < S, smallest terms first; K in chunks of 256 (exact FP32 sums per chunk)
  for (int lvl = slices - 1; lvl >= 0; --lvl) {
    for (int s = 0; s <= lvl; ++s) {
      const int t = lvl - s;
      for (int k0 = 0; k0 < K; k0 += 256) {
        k_tc_gemm<1><<<dim3(M / TM, N / TN), TC_THREADS, 2 * TILE_BYTES, stream>>>(
            sa + (int64_t)s * M * K + k0, sb + (int64_t)t * N * K + k0, 256, K, K, nullptr, 0, C, N, ea, eb,
            -8 * (s + t + 2), err);
      }
    }
  }
  return cudaPeekAtLastError() == cudaSuccess ? SKN_OK : SKN_ERR_CUDA;
}
