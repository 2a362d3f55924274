// skn_eigh_gen_vectors_noalloc: eigenvalues and eigenvectors with no device
// allocation by the caller or the library.
//
// The kernels are those of eigh.cu (included below for their code alone, with
// the default 128-thread launch shape).  Their scratch -- the two queue
// counters, the tridiagonal/tau rows and the inverse-iteration workspace --
// lives in one file-scope __device__ array of fixed size instead of buffers
// the caller passes.  The array is set aside when the CUDA module holding this
// file is loaded on a device; with lazy module loading (the CUDA runtime's
// default) that happens inside the first call on that device, which is why
// callers make one call (n_prob = 0 is enough) at start-up.  Every call looks
// up the array's device address on the current device: the lookup is cheap
// once the module is loaded, and an address kept from an earlier context
// would be stale after cudaDeviceReset.
#define SKN_EIG_KERNELS_ONLY
#define SKN_EIG_NS_TAG _noalloc
#include "eigh.cu"

namespace {

constexpr int64_t NA_COUNTER_DOUBLES = 32;   // 256 bytes: the two queue counters, then padding
constexpr int64_t NA_TRI_DOUBLES = 4 * (int64_t)SKN_NOALLOC_MAX_ROWS;
constexpr int64_t NA_SCRATCH_DOUBLES = SKN_NOALLOC_SCRATCH_DOUBLES;
constexpr int64_t NA_TOTAL_DOUBLES = NA_COUNTER_DOUBLES + NA_TRI_DOUBLES + NA_SCRATCH_DOUBLES;
static_assert(SKN_NOALLOC_MAX_N <= MAX_N, "the static variant cannot exceed the eigensolver's bound");
static_assert(NA_TRI_DOUBLES % 32 == 0, "keep the scratch section 256-byte aligned");
static_assert((int64_t)5 * SKN_NOALLOC_MAX_N * VNT <= NA_SCRATCH_DOUBLES, "one vector CTA must fit");

// [counters | tri: 4 doubles per eigenvalue row | inverse-iteration scratch]
static __device__ __align__(256) double g_noalloc[NA_TOTAL_DOUBLES];

// Device address of g_noalloc on the current device.  In host code the name g_noalloc is a host-side
// stand-in, not a device address, so kernels get only what this lookup returns.
cudaError_t noalloc_base(double** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc);
  if (e != cudaSuccess) return e;
  *out = static_cast<double*>(p);
  return cudaSuccess;
}

}  // namespace

extern "C" int skn_eigh_gen_vectors_noalloc(int n_prob, const int32_t* n, const int64_t* hs_off,
                                            const int64_t* eig_off, const int32_t* order, double* H, double* S,
                                            double* eig, double* vec, int32_t* status, int64_t n_rows, int max_n,
                                            cudaStream_t stream) {
  if (n_prob < 0 || max_n < 0 || n_rows < 0) return SKN_ERR_ARG;
  // the lookup comes first so that a call with no problems loads the module on this device (a warm-up)
  double* base = nullptr;
  if (noalloc_base(&base) != cudaSuccess) return SKN_ERR_CUDA;
  if (n_prob == 0) return SKN_OK;
  if (!n || !hs_off || !eig_off || !order || !H || !S || !eig || !vec || !status) return SKN_ERR_ARG;
  if (max_n > SKN_NOALLOC_MAX_N || n_rows > SKN_NOALLOC_MAX_ROWS) return SKN_ERR_CAPACITY;
  int32_t* counter = reinterpret_cast<int32_t*>(base);
  double* tri = base + NA_COUNTER_DOUBLES;
  double* scratch = tri + NA_TRI_DOUBLES;

  const int mn = max_n < 1 ? 1 : max_n;
  const int use_smem_mats = 1;
  if (set_smem_limit_once() != cudaSuccess) return SKN_ERR_CUDA;
  int per_sm = 0, dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t smem = eig_smem_bytes(mn);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_eigh_gen<false>, NT, smem) != cudaSuccess ||
      per_sm < 1)
    return SKN_ERR_CUDA;
  int grid = sms * per_sm;
  if (grid > n_prob) grid = n_prob;
  // the vector stage takes as many CTAs as the fixed workspace holds (at most 2 per SM)
  int vgrid = (int)(NA_SCRATCH_DOUBLES / ((int64_t)5 * mn * VNT));
  if (vgrid > 2 * sms) vgrid = 2 * sms;
  if (vgrid > n_prob) vgrid = n_prob;
  // only the queue counters must start at zero; every tri row and scratch entry is written before it is read
  if (cudaMemsetAsync(counter, 0, 2 * sizeof(int32_t), stream) != cudaSuccess) return SKN_ERR_CUDA;
  k_eigh_gen<false><<<grid, NT, smem, stream>>>(n_prob, n, hs_off, eig_off, order, (double2*)H, (double2*)S, eig, status,
                                         counter, mn, use_smem_mats, tri, n_rows);
  if (cudaPeekAtLastError() != cudaSuccess) return SKN_ERR_CUDA;
  k_eigvec<<<vgrid, VNT, vec_smem_bytes(mn), stream>>>(n_prob, n, hs_off, eig_off, order, (const double2*)H,
                                                       (const double2*)S, eig, tri, status, (double2*)vec, scratch,
                                                       counter + 1, mn);
  return cudaPeekAtLastError() == cudaSuccess ? SKN_OK : SKN_ERR_CUDA;
}
