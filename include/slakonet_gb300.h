/*
 * slakonet_gb300.h -- C ABI of the GB300 (sm_103a) SlakoNet electronic-structure path.
 *
 * Every entry point takes raw device pointers owned by the caller, sizes, and
 * a cudaStream_t; work is stream-ordered and the functions return an int
 * status (SKN_OK == 0).  No entry point allocates device memory, throws, or
 * synchronises the host unless its comment says so.  Per-problem numerical
 * failures (S(k) not positive definite, NaN, no Fermi convergence) are
 * reported in caller-provided status arrays, never as a failed call.
 *
 * Units: Bohr and Hartree; complex numbers are interleaved (re, im) doubles.
 * Matrices are column-major, one n x n block per (structure, k) problem.
 *
 * Each declaration names the part of the reference SlakoNet code it
 * replaces (paths relative to the reference project).
 */
#ifndef SLAKONET_GB300_H
#define SLAKONET_GB300_H

#include <stdint.h>
#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  SKN_OK = 0,
  SKN_ERR_ARG = 1,          /* invalid argument (null pointer, bad size)          */
  SKN_ERR_NOT_SPD = 2,      /* per-problem status: S(k) not positive definite      */
  SKN_ERR_NAN = 3,          /* per-problem status: NaN met                         */
  SKN_ERR_NO_CONVERGE = 4,  /* per-structure status: Fermi search hit max_iter     */
  SKN_ERR_CAPACITY = 5,     /* request larger than the kernel's supported size     */
  SKN_ERR_CUDA = 6          /* a CUDA launch or runtime call failed                */
};

/* Version of this ABI (major * 100 + minor). */
int skn_abi_version(void);

/* Maximum orbitals per atom (spdf = 16) and shells per atom supported. */
#define SKN_MAX_ORB_PER_ATOM 16
#define SKN_MAX_SHELLS 4
/* Number of doubles per structure in the skn_fermi_gap statistics record. */
#define SKN_NSTAT 24

/*
 * Bond counting.  Replaces the periodic image/distance tables of
 * Periodic.get_cell_translations / _periodic_distance
 * (slakonet/atoms.py:165-243) and the 0 < d < cutoff mask of hs_matrix
 * (slakonet/slaterkoster.py:269-276).
 *   atom_ptr[n_struct+1]   atoms of structure s are atom_ptr[s] .. atom_ptr[s+1)-1
 *   positions[3*A]         Cartesian positions (Bohr)
 *   cells[9*n_struct]      row-major lattice vectors (row i = vector i, Bohr)
 *   image_range[3*n_struct] half widths r: translations T in [-r, r]^3
 *   n_pairs                total ordered atom pairs, sum over structures of N_s^2
 *   pair_base[n_struct]    first atom-pair slot of structure s (sum of N^2 before s)
 *   pair_counts[n_pairs]   out: bonds of ordered pair (i, j) at pair_base[s] + i*N + j
 */
int skn_bond_counts(int n_struct, int64_t n_pairs, const int32_t* atom_ptr, const double* positions,
                    const double* cells, const int32_t* image_range, double cutoff,
                    const int64_t* pair_base, int32_t* pair_counts, cudaStream_t stream);

/*
 * Bond table fill: writes every directed bond (i, j, T) with 0 < d < cutoff,
 * ordered by (structure, i, j, T with x slowest).  Same inputs as
 * skn_bond_counts plus
 *   pair_ptr[P]            exclusive scan of pair_counts (first bond of each pair)
 *   pair_blk_base[P]       first block double of each pair's bonds
 *   atom_norb[A]           orbitals per atom
 * Outputs per bond: bond_i, bond_j (global atom index), bond_img (linear
 * index of T in the structure's (2r+1)^3 box, x slowest), bond_d (Bohr),
 * bond_u[3] (unit vector i -> j + T), bond_blk (offset of its real-space
 * block, column-major norb_i x norb_j).
 */
int skn_bond_fill(int n_struct, int64_t n_pairs, const int32_t* atom_ptr, const double* positions,
                  const double* cells, const int32_t* image_range, double cutoff,
                  const int64_t* pair_base, const int64_t* pair_ptr, const int64_t* pair_blk_base,
                  const int32_t* atom_norb, int32_t* bond_i, int32_t* bond_j, int32_t* bond_img,
                  double* bond_d, double* bond_u, int64_t* bond_blk, cudaStream_t stream);

/*
 * Bloch phases exp(i 2 pi k . T) for every (k, T) of each structure's box.
 * Replaces Periodic.phase (slakonet/atoms.py:543-558).
 *   k_ptr[n_struct+1]      k-points of structure s are k_ptr[s] .. k_ptr[s+1)-1
 *   kpoints[3*K]           fractional k
 *   phase_base[n_struct]   first phase of structure s; layout [nk_s][n_img_s]
 *   phases[2*...]          out, complex
 */
int skn_image_phases(int n_struct, const int32_t* image_range, const int32_t* k_ptr,
                     const double* kpoints, const int64_t* phase_base, double* phases,
                     cudaStream_t stream);

/*
 * Real-space Slater-Koster blocks H(R), S(R) for every bond: spline lookup
 * of the integrals and rotation into the crystal frame.  Replaces
 * _gather_off_site / SkfFeed.off_site / PolyInterpU (slakonet/slaterkoster.py:834-946,
 * slakonet/skfeed.py:285-326, slakonet/interpolation.py:107-311) and
 * sub_block_rot / sub_block_ref (slakonet/slaterkoster.py:1013-1122).
 *   atom_species[A]        species index of each atom
 *   sp_nshell[nsp], sp_shell_l[4*nsp], sp_norb[nsp]   shell layout per species
 *   tab_index[16*nsp*nsp]  table of (spA, spB, l1, l2) at ((spA*nsp+spB)*4+l1)*4+l2, -1 if absent (l1 <= l2)
 *   tab_off[ntab], tab_ngrid[ntab], tab_step[ntab]    table t: (l1+1) rows of tab_ngrid doubles
 *                          at tab_H + tab_off[t] (and tab_S + tab_off[t]); row r is bond order r,
 *                          column g the value at (g+1)*tab_step
 *   blk_H, blk_S           out: real-space blocks at bond_blk[b]
 *   status                 out (device int): SKN_ERR_ARG if a needed table is missing
 */
int skn_sk_blocks(int64_t n_bonds, const int32_t* bond_i, const int32_t* bond_j,
                  const double* bond_d, const double* bond_u, const int64_t* bond_blk,
                  const int32_t* atom_species, int n_species, const int32_t* sp_nshell,
                  const int32_t* sp_shell_l, const int32_t* sp_norb, const int32_t* tab_index,
                  const int64_t* tab_off, const int32_t* tab_ngrid, const double* tab_step,
                  const double* tab_H, const double* tab_S, double* blk_H, double* blk_S,
                  int32_t* status, cudaStream_t stream);

/*
 * Bloch sums H(k) = onsite + sum_T H(T) exp(i 2 pi k . T), same for S, as
 * dense column-major matrices.  Replaces _pe_sk_data2 and the block scatter
 * of hs_matrix (slakonet/slaterkoster.py:327-439, 971-1010).
 * Problems p = (structure prob_struct[p], k index prob_k[p]) write
 * n_s x n_s complex matrices at hs_off[p] (complex elements).
 *   atom_ptr, pair_base, pair_ptr as above; orb_ptr[n_struct+1] orbital range of s;
 *   orb_atom[n_orb_total]  local atom index of each orbital; atom_orb_off[A] first
 *                          local orbital of each atom; atom_norb[A];
 *   onsite_H[n_orb_total]  diagonal on-site energies (S gets 1)
 */
int skn_bloch(int n_prob, const int32_t* prob_struct, const int32_t* prob_k, const int64_t* hs_off,
              const int32_t* atom_ptr, const int32_t* orb_ptr, const int32_t* orb_atom,
              const int32_t* atom_orb_off, const int32_t* atom_norb, const int64_t* pair_base,
              const int64_t* pair_ptr, const int32_t* bond_img, const int64_t* bond_blk,
              const double* blk_H, const double* blk_S, const int32_t* image_range,
              const int64_t* phase_base, const double* phases, const double* onsite_H,
              int max_n, double* H, double* S, cudaStream_t stream);

/*
 * The same Bloch sums organised by atom pair: a warp per (ordered atom pair,
 * chunk of 8 k-points), its lanes over (k-point, block element), so warps
 * stay full when blocks are small (1x1, 1x4, 4x4 orbitals) and a small cell's
 * many k-points spread over many warps; the warps of a CTA take the adjacent
 * row blocks of one column block, so columns are written in long runs.
 * Values are bitwise those of skn_bloch.  Replaces the same reference code as
 * skn_bloch.
 *   n_struct               structures
 *   n_units, unit_base[n_struct]   work units, numbered from unit_base[s]
 *                          (exclusive prefix sum): structure s owns
 *                          ceil(nk_s / 8) * N_s^2 of them with lower = 0 and
 *                          ceil(nk_s / 8) * N_s (N_s + 1) / 2 with lower = 1
 *   k_ptr[n_struct+1]      problem index of each structure's first k-point (problems
 *                          of a structure are consecutive, k-point order)
 *   lower                  1: write only the entries on or below the diagonal (what the
 *                          eigensolvers read; the strict upper triangle is left as it
 *                          was), 0: the full matrices
 * Other arguments as skn_bloch.
 */
int skn_bloch_pairs(int n_struct, int64_t n_units, const int64_t* unit_base, const int32_t* k_ptr,
                    const int64_t* hs_off, const int32_t* atom_ptr, const int32_t* orb_ptr,
                    const int32_t* atom_orb_off, const int32_t* atom_norb, const int64_t* pair_base,
                    const int64_t* pair_ptr, const int32_t* bond_img, const int64_t* bond_blk, const double* blk_H,
                    const double* blk_S, const int32_t* image_range, const int64_t* phase_base, const double* phases,
                    const double* onsite_H, int lower, double* H, double* S, cudaStream_t stream);

/*
 * Batched generalized Hermitian eigenvalues H x = e S x, one problem per
 * (structure, k).  Cholesky S = L L^H, reduction C = L^-1 H L^-H,
 * Householder tridiagonalisation, Sturm bisection; FP64 throughout.
 * Replaces eighb(..., scheme="chol") and the per-k loop of
 * SimpleDftb.__call__ (slakonet/utils.py:741-783, slakonet/main.py:137-196).
 *   n[p], hs_off[p], eig_off[p]  size and offsets of problem p
 *   order[n_prob]          processing order (largest first is best)
 *   H, S                   in/out: overwritten by the factorisations
 *   eig                    out: ascending eigenvalues (Hartree) at eig_off[p]
 *   status[p]              out: SKN_OK, SKN_ERR_NOT_SPD or SKN_ERR_NAN
 *   work_counter           device int scratch, zeroed by the call (stream-ordered)
 *   max_n                  largest n[p]
 */
int skn_eigh_gen_batched(int n_prob, const int32_t* n, const int64_t* hs_off, const int64_t* eig_off,
                         const int32_t* order, double* H, double* S, double* eig, int32_t* status,
                         int32_t* work_counter, int max_n, cudaStream_t stream);

/*
 * skn_eigh_gen_batched for problems whose H and S are real symmetric (every
 * imaginary part zero, e.g. the Bloch sums at k-points with 2k integer):
 * only the real parts are read and written, in real arithmetic (a quarter of
 * the FP64 work).  The steps are those of skn_eigh_gen_batched minus terms
 * that are exactly zero for real input, so the eigenvalues are the same.
 * Imaginary parts are ignored, not checked: route only real problems here.
 */
int skn_eigh_gen_batched_real(int n_prob, const int32_t* n, const int64_t* hs_off, const int64_t* eig_off,
                              const int32_t* order, double* H, double* S, double* eig, int32_t* status,
                              int32_t* work_counter, int max_n, cudaStream_t stream);

/*
 * Eigenvalues and eigenvectors of the same batched problems.  Replaces the
 * eigenvector output of eighb (slakonet/utils.py:741-783) that
 * SimpleDftb.__call__ keeps with with_eigenvectors (slakonet/main.py:137-196).
 * Runs the values kernel keeping the reflectors, tau and the tridiagonal,
 * then inverse iteration on the tridiagonal (clusters re-orthogonalised),
 * the Householder back-transformation and x = L^-H y, so x^H S x = 1.
 *   vec       out: complex, problem p at hs_off[p]; vec[i*n + j] = component i of eigenvector j
 *   tri       scratch: 4 * sum(n) doubles (d, e, tau per problem at 4*eig_off[p])
 *   scratch   scratch: skn_eigh_vectors_scratch_bytes(n_prob, max_n) bytes
 *   work_counter  device int[2] scratch
 * H and S are left holding the reflectors and L.
 */
int skn_eigh_gen_vectors(int n_prob, const int32_t* n, const int64_t* hs_off, const int64_t* eig_off,
                         const int32_t* order, double* H, double* S, double* eig, double* vec, int32_t* status,
                         double* tri, double* scratch, int64_t scratch_bytes, int32_t* work_counter, int max_n,
                         cudaStream_t stream);

/* Host-side query: bytes of `scratch` skn_eigh_gen_vectors needs (written to *bytes). */
int skn_eigh_vectors_scratch_bytes(int n_prob, int max_n, int64_t* bytes);

/*
 * skn_eigh_gen_vectors without any device allocation: no counterpart in the
 * reference (which allocates through torch on every call).  For callers that
 * cannot allocate device memory: a host binding that receives only device
 * pointers from another runtime and owns no allocator, or a latency-bound
 * service that keeps cudaMalloc/cudaFree (which can synchronise the device or
 * fail under memory pressure) out of its request path.
 * Same outputs, same contract, minus tri, scratch and work_counter: those live
 * in one fixed library-owned device array (about 40 MiB per device), held by
 * every device that loads the library until the process exits.
 *   n_rows   length of eig = sum of n[p] (every eig_off[p] + n[p] <= n_rows)
 * Limits: max_n <= SKN_NOALLOC_MAX_N and n_rows <= SKN_NOALLOC_MAX_ROWS, else
 * SKN_ERR_CAPACITY and nothing is launched.  On the device, a problem with
 * n[p] > max_n or eig_off[p] + n[p] > n_rows is skipped with status[p] =
 * SKN_ERR_CAPACITY and its outputs untouched, so an understated n_rows cannot
 * write past the fixed array.  The vector stage runs on as many CTAs as the
 * fixed workspace holds (up to 2 per SM), so large batches are slower than
 * with skn_eigh_gen_vectors.
 * The array is set aside when the library's CUDA module is loaded on a device;
 * with lazy module loading (the CUDA default) that is the first call on that
 * device, so make one call at start-up (n_prob = 0 is enough), before any
 * stream capture.  Every call looks up the array's device address on the
 * current device.  Calls share the array, which keeps the last call's
 * contents: two calls in flight at once on one device (other streams or host
 * threads) race and corrupt each other; order them on one stream or serialise
 * them.
 */
#define SKN_NOALLOC_MAX_N 512
#define SKN_NOALLOC_MAX_ROWS 262144             /* 8 MiB of tridiagonal rows            */
#define SKN_NOALLOC_SCRATCH_DOUBLES 4194304     /* 32 MiB of inverse-iteration scratch  */
int skn_eigh_gen_vectors_noalloc(int n_prob, const int32_t* n, const int64_t* hs_off, const int64_t* eig_off,
                                 const int32_t* order, double* H, double* S, double* eig, double* vec,
                                 int32_t* status, int64_t n_rows, int max_n, cudaStream_t stream);

/*
 * Eigenvalues of large problems, one thread-block cluster per problem.
 * Replaces the same eighb call as skn_eigh_gen_batched (slakonet/utils.py:
 * 741-783) for problems that are too slow on one SM or too large for its
 * shared memory (n > 2048).  Same steps, results to rounding: `cluster` CTAs
 * (1..16, one per SM) split every O(n^2)-per-column loop of the Cholesky,
 * reduction and tridiagonalisation and the bisection, with cluster barriers
 * between phases.  Arguments as skn_eigh_gen_batched, plus
 *   scratch   device scratch of skn_eigh_large_scratch_bytes(n_prob, max_n, cluster) bytes
 *   cluster   CTAs per problem (more than 8 uses the non-portable cluster size)
 * max_n <= 9216 (the tridiagonal is bisected from shared memory), else
 * SKN_ERR_CAPACITY; SKN_ERR_CAPACITY also when no cluster of that size fits.
 */
int skn_eigh_gen_large(int n_prob, const int32_t* n, const int64_t* hs_off, const int64_t* eig_off,
                       const int32_t* order, double* H, double* S, double* eig, int32_t* status,
                       int32_t* work_counter, double* scratch, int64_t scratch_bytes, int max_n, int cluster,
                       cudaStream_t stream);
/* Host-side query: bytes of `scratch` skn_eigh_gen_large needs (written to *bytes). */
int skn_eigh_large_scratch_bytes(int n_prob, int max_n, int cluster, int64_t* bytes);

/*
 * Eigenvalues of large problems with the whole GPU: blocked (32-column panels)
 * Cholesky, zhegst-order reduction and zlatrd-order tridiagonalisation, each
 * step one kernel launch across all problems of the group, with tiled rank-2k
 * updates and a tiled Hermitian matrix-vector product, then Sturm-count
 * eigenvalues.  Replaces the same eighb call as skn_eigh_gen_batched
 * (slakonet/utils.py:741-783) for problems too large for one SM, without the
 * cluster path's bound of 16 SMs per problem.  The host issues about 6n + 9n/32
 * launches on `stream`, so it suits problems of more than ~1000 orbitals.
 *   n_prob    problems in the group (<= 32767); all must have n orbitals
 *   n         orbitals of every problem (host value, 1..32768)
 *   prob      [n_prob] (device) problem index of each group slot, into the arrays below
 *   nvec, hs_off, eig_off, H, S, eig, status   as skn_eigh_gen_batched; a problem
 *             whose nvec differs from n gets SKN_ERR_CAPACITY and is not touched
 *   scratch   device scratch of skn_eigh_wide_scratch_bytes(n_prob, n) bytes
 *   real      1 when every problem's H and S are exactly real (their imaginary
 *             parts are then neither read nor written), else 0
 * Results depend only on each problem: every cross-CTA sum is reduced in a
 * fixed order.  H and S are overwritten; the upper triangles are not read.
 */
int skn_eigh_gen_wide(int n_prob, int n, const int32_t* prob, const int32_t* nvec, const int64_t* hs_off,
                      const int64_t* eig_off, double* H, double* S, double* eig, int32_t* status, double* scratch,
                      int64_t scratch_bytes, int real, cudaStream_t stream);
/* Host-side query: bytes of `scratch` skn_eigh_gen_wide needs (written to *bytes). */
int skn_eigh_wide_scratch_bytes(int n_prob, int n, int64_t* bytes);
/*
 * skn_eigh_gen_wide with its rank-2k trailing updates (Cholesky, reduction
 * and tridiagonalisation panels, trailing matrices of 512 rows and more) on
 * the bf16 tensor cores (tcgen05, TMEM accumulators), FP64-accurate by
 * error-free splitting: every row of the update's operands is split into 7
 * integer slices of 7 bits, slice products of one level accumulate exactly in
 * FP32, and the levels are combined exactly before one FP64 rounding.  Same
 * arguments, scratch and contract as skn_eigh_gen_wide; a tensor-core stage
 * whose completion wait runs out sets the problem's status to SKN_ERR_CUDA.
 * No reference counterpart beyond the eighb call skn_eigh_gen_wide replaces.
 */
int skn_eigh_gen_wide_tc(int n_prob, int n, const int32_t* prob, const int32_t* nvec, const int64_t* hs_off,
                         const int64_t* eig_off, double* H, double* S, double* eig, int32_t* status, double* scratch,
                         int64_t scratch_bytes, int real, cudaStream_t stream);

/*
 * The same eigensolver compiled in more launch shapes: 32 threads per CTA with
 * up to 16 CTAs per SM (suffix _t32), 64 threads with up to 8 (_t64), 256
 * threads with up to 3 (_t256), and 128 threads with up to 3 whose Cholesky and
 * reduction run in 32-column panels (_blk).  The unsuffixed entry points use
 * 128 threads and up to 5 CTAs per SM.  Contracts are identical.  The project's
 * autotuner (slakonet_gb300/autotune.py) picks a shape per problem-size bucket.
 * Each shape exports the four entry points below with its suffix; the _t64 and
 * _t256 ones are spelled out.
 */
int skn_eigh_gen_batched_t64(int n_prob, const int32_t* n, const int64_t* hs_off, const int64_t* eig_off,
                             const int32_t* order, double* H, double* S, double* eig, int32_t* status,
                             int32_t* work_counter, int max_n, cudaStream_t stream);
int skn_eigh_gen_batched_t256(int n_prob, const int32_t* n, const int64_t* hs_off, const int64_t* eig_off,
                              const int32_t* order, double* H, double* S, double* eig, int32_t* status,
                              int32_t* work_counter, int max_n, cudaStream_t stream);
int skn_eigh_gen_vectors_t64(int n_prob, const int32_t* n, const int64_t* hs_off, const int64_t* eig_off,
                             const int32_t* order, double* H, double* S, double* eig, double* vec, int32_t* status,
                             double* tri, double* scratch, int64_t scratch_bytes, int32_t* work_counter, int max_n,
                             cudaStream_t stream);
int skn_eigh_gen_vectors_t256(int n_prob, const int32_t* n, const int64_t* hs_off, const int64_t* eig_off,
                              const int32_t* order, double* H, double* S, double* eig, double* vec,
                              int32_t* status, double* tri, double* scratch, int64_t scratch_bytes,
                              int32_t* work_counter, int max_n, cudaStream_t stream);
int skn_eigh_gen_batched_real_t64(int n_prob, const int32_t* n, const int64_t* hs_off, const int64_t* eig_off,
                                  const int32_t* order, double* H, double* S, double* eig, int32_t* status,
                                  int32_t* work_counter, int max_n, cudaStream_t stream);
int skn_eigh_gen_batched_real_t256(int n_prob, const int32_t* n, const int64_t* hs_off, const int64_t* eig_off,
                                   const int32_t* order, double* H, double* S, double* eig, int32_t* status,
                                   int32_t* work_counter, int max_n, cudaStream_t stream);
int skn_eigh_vectors_scratch_bytes_t64(int n_prob, int max_n, int64_t* bytes);
int skn_eigh_vectors_scratch_bytes_t256(int n_prob, int max_n, int64_t* bytes);

/*
 * Atom-type projected DOS of one structure.  Replaces
 * compute_atom_projected_dos (slakonet/predict_slakonet.py:119-210).
 *   eig        [nk][nb] eigenvalues, Hartree
 *   vec        complex [nk][n_orb][nb]: component i of eigenvector b (x^H S x = 1)
 *   orb_group  [n_orb] atom-type index (0..n_group-1) of each orbital
 *   fermi_ev   Fermi level (eV); the grid is linspace(e_lo, e_hi, npts) eV relative to it
 *   sigma      Gaussian width (eV); h2e the Hartree-to-eV factor of the eigenvalues
 *   weights    scratch: nk * nb * n_group doubles
 *   grid       out: [npts]; pdos out: [n_group][npts]
 * pdos[g][e] = (1/nk) sum_{k,b} (sum_{i in g} |c_ib|^2) exp(-((E_e + E_F - e_kb h2e)/sigma)^2 / 2) / (sigma sqrt(2 pi)).
 */
int skn_atom_pdos(int nk, int nb, int n_orb, const double* eig, const double* vec, const int32_t* orb_group,
                  int n_group, double fermi_ev, double e_lo, double e_hi, int npts, double sigma, double h2e,
                  double* weights, double* grid, double* pdos, cudaStream_t stream);

/*
 * Fermi level, band gap and band-structure statistics per structure.
 * Replaces fermi_search / fermi_dirac (slakonet/fermi.py:139-215),
 * calculate_band_gap (slakonet/main.py:637-707),
 * calculate_band_structure_properties (slakonet/main.py:1539-1642) and
 * the get_fermi extras of compute_multi_element_properties (slakonet/optim.py:1011-1060).
 *   eig_off[s], nk[s], nb[s]   eigenvalues [nk][nb] of structure s (ascending per k)
 *   kw_off[s], kweights        k weights of structure s
 *   nelec[s]                   electron count
 *   mu[s] out; stats[SKN_NSTAT*s] out (layout in slakonet_gb300/engine.py STAT_*);
 *   status[s] out: SKN_OK or SKN_ERR_NO_CONVERGE (NaN propagates as in the reference)
 */
int skn_fermi_gap(int n_struct, const int64_t* eig_off, const int32_t* nk, const int32_t* nb,
                  const int64_t* kw_off, const double* kweights, const double* nelec, const double* eig,
                  double kT, double tol, int max_iter, double* mu, double* stats, int32_t* status,
                  cudaStream_t stream);

/*
 * Gaussian density of states on a uniform grid, energies shifted by the
 * Fermi level and in eV.  Replaces calculate_dos and the DOS block of
 * get_properties_dict (slakonet/main.py:709-797, 1766-1800).
 * dos[s*npts + i] = sum_k w_k sum_b exp(-((E_i - (e_kb - mu_s) H2E)/sigma)^2/2)/(sigma sqrt(2 pi)).
 * window_sigmas > 0 skips terms beyond that many sigmas (each skipped term
 * is below exp(-window^2/2)); 0 sums every term.  Also fills grid[npts]
 * and stats entries 16..18 (dos_at_fermi, gap centre, trapezoid total).
 */
int skn_dos(int n_struct, const int64_t* eig_off, const int32_t* nk, const int32_t* nb,
            const int64_t* kw_off, const double* kweights, const double* eig, const double* mu,
            double e_lo, double e_hi, int npts, double sigma, double window_sigmas,
            double* grid, double* dos, double* stats, cudaStream_t stream);

/*
 * Adjoint, step 1: weighted eigenvector projectors per problem,
 *   G_ab = sum_n g_n conj(c_n[a]) c_n[b],  F_ab = sum_n g_n e_n conj(c_n[a]) c_n[b],
 * from eigenvectors `vec` (skn_eigh_gen_vectors layout), eigenvalues and
 * grad_eig = dL/de; G, F column-major complex at hs_off[p] (zero where
 * status[p] != SKN_OK; status may be NULL).  With these,
 * dL/dH(k) = G and dL/dS(k) = -F.  Replaces the eigenvalue part of
 * _SymEigB.backward (slakonet/utils.py:387-473), whose complex case omits
 * the conjugate of the eigenvectors.
 */
int skn_adj_projectors(int n_prob, const int32_t* n, const int64_t* hs_off, const int64_t* eig_off,
                       const double* vec, const double* eig, const double* grad_eig, const int32_t* status,
                       double* G, double* F, cudaStream_t stream);

/*
 * Adjoint, step 2: dL/dB for every bond's real-space H and S block,
 * dL/dB_ab(T) = sum_k Re(G_ab(k) exp(i 2 pi k.T)) (S: -F), written in the
 * block layout of skn_sk_blocks.  The autograd counterpart is the backward of
 * _pe_sk_data2's phase multiply and scatter (slakonet/slaterkoster.py:971-1010).
 *   atom_struct[A], struct_prob0[S] (first problem of each structure; a
 *   structure's problems are consecutive, k-ordered), nk[S], nb[S].
 */
int skn_adj_bloch(int64_t n_bonds, const int32_t* bond_i, const int32_t* bond_j, const int32_t* bond_img,
                  const int64_t* bond_blk, const int32_t* atom_struct, const int32_t* atom_orb_off,
                  const int32_t* atom_norb, const int32_t* struct_prob0, const int32_t* nk, const int32_t* nb,
                  const int64_t* hs_off, const int32_t* image_range, const int64_t* phase_base, const double* phases,
                  const double* G, const double* F, double* grad_blk_H, double* grad_blk_S, cudaStream_t stream);

/*
 * Adjoint, step 3: pull the block gradients back through the rotation and
 * the 8-point spline (or the tail functional) onto the packed tables,
 * accumulating into grad_tab_H / grad_tab_S (same layout as tab_H / tab_S;
 * zero them first).  The autograd counterpart is the backward of
 * sub_block_rot and PolyInterpU (slakonet/slaterkoster.py:1013-1122,
 * slakonet/interpolation.py:107-311).
 */
int skn_adj_tables(int64_t n_bonds, const int32_t* bond_i, const int32_t* bond_j, const double* bond_d,
                   const double* bond_u, const int64_t* bond_blk, const int32_t* atom_species, int n_species,
                   const int32_t* sp_nshell, const int32_t* sp_shell_l, const int32_t* sp_norb,
                   const int32_t* tab_index, const int64_t* tab_off, const int32_t* tab_ngrid, const double* tab_step,
                   const double* grad_blk_H, const double* grad_blk_S, double* grad_tab_H, double* grad_tab_S,
                   cudaStream_t stream);

/*
 * DOS backward: grad_eig[e] += dL/de from grad_dos = dL/dDOS of skn_dos with
 * the same grid arguments (mu held fixed, as the reference detaches it in
 * fermi_search, slakonet/fermi.py:191-196).  max_count = max over
 * structures of nk * nb.
 */
int skn_dos_backward(int n_struct, const int64_t* eig_off, const int32_t* nk, const int32_t* nb,
                     const int64_t* kw_off, const double* kweights, const double* eig, const double* mu,
                     double e_lo, double e_hi, int npts, double sigma, double window_sigmas,
                     const double* grad_dos, double* grad_eig, int max_count, cudaStream_t stream);

/*
 * FP64 fused multiply-add throughput probe (no counterpart in the reference):
 * blocks x 256 threads, 8 independent FMA chains of `iters` steps each,
 * 16 * iters flops per thread, result written to out[blocks*256].  Used to
 * measure the FP64 roofline the eigensolver is bound by.
 */
int skn_fp64_probe(double* out, int blocks, int iters, cudaStream_t stream);

/*
 * The same measurement on the FP64 tensor instruction (mma.sync m8n8k4 f64):
 * `blocks` CTAs of 256 threads, each warp running 8 independent chains of
 * `iters` instructions (512 flops each per warp), `out` holds blocks*256
 * doubles.  No reference counterpart: it shows whether FP64 tensor MMA is
 * faster than FP64 FMA on this GPU, which decides how the eigensolver's
 * updates are shaped.
 */
int skn_fp64_probe_dmma(double* out, int blocks, int iters, cudaStream_t stream);

/*
 * bf16 tensor-core GEMM (tcgen05, TMEM accumulators), no reference
 * counterpart: D[M x N] = A B^T in FP32, A [M x K] and B [N x K] bf16 with K
 * contiguous (raw bf16 bit patterns), D row-major.  M and N multiples of 128,
 * K a multiple of 64, pointers 16-byte aligned (else SKN_ERR_ARG).  *err is
 * set to 1 when a stage's completion wait exceeded its iteration limit.  The
 * building block of the FP64 emulation below; with integer operands of at
 * most 8 significant bits and K <= 256 every product and partial sum is an
 * integer below 2^24, which an exact FP32 accumulator holds without rounding.
 */
int skn_tc_gemm_bf16(const uint16_t* A, const uint16_t* B, float* D, int M, int N, int K, int32_t* err,
                     cudaStream_t stream);

/*
 * FP64 GEMM C[M x N] = A B^T (A [M x K], B [N x K], FP64 row-major, K
 * contiguous) computed on the bf16 tensor cores by error-free splitting into
 * `slices` (1..8) integer bf16 slices per operand row (Ozaki, Ogita and
 * Oishi 2012): the slice products with s + t < slices, each exact in FP32 for
 * K chunks of 256, are scaled by powers of two and summed in FP64.  With 7
 * slices the result agrees with an FP64 GEMM to FP64 rounding.  No reference
 * counterpart: GB300's FP64 tensor instruction runs no faster than FP64 FMA,
 * so this is the tensor-core route for the eigensolver's GEMM-shaped FP64
 * updates.  M, N multiples of 128, K a multiple of 256.
 *   scratch  device buffer of skn_gemm_f64_emulated_scratch_bytes bytes
 */
int skn_gemm_f64_emulated(const double* A, const double* B, double* C, int M, int N, int K, int slices,
                          void* scratch, int64_t scratch_bytes, int32_t* err, cudaStream_t stream);
/* Host-side query: scratch bytes skn_gemm_f64_emulated needs (written to *bytes). */
int skn_gemm_f64_emulated_scratch_bytes(int M, int N, int K, int slices, int64_t* bytes);

#ifdef __cplusplus
}
#endif
#endif /* SLAKONET_GB300_H */
