/*
 * qimpy_gb300: GB300 (sm_103a) plane-wave Hamiltonian apply for QimPy's eigensolvers.
 *
 * Plain C ABI.  Every pointer argument is a device pointer unless stated
 * otherwise; complex arrays are interleaved (re, im) like C99 `double complex`
 * / torch complex128 (QGB_F64) or `float complex` / complex64 (QGB_F32).
 * Every call is asynchronous on `stream` (a cudaStream_t passed as void*;
 * NULL = legacy default stream), performs no host synchronisation and no
 * device allocation, and returns 0 on success or a QGB_ERR_* code; the text
 * of the last error on the calling thread is returned by qgb_last_error().
 *
 * Array layouts (the reference's Wavefunction.coeff (spin, k, band, spinor,
 * basis) with the singleton spin and spinor axes dropped):
 *   C, HC   [nk][nb][n_tot]      wavefunction coefficients, padded basis
 *   beta    [nk][P][n_tot]       projectors beta_p(k+G); padding must be zero
 *   projT   [nk][nb][P]          projections <beta_p|psi_b> (band-major)
 *   D       [n_atoms][pa][pa]    per-atom blocks of the block-diagonal D_all,
 *                                row-major, complex, P = n_atoms * pa
 * Input wavefunctions must have zero padding (entries g >= n[k]), the
 * invariant Wavefunction.constrain() keeps in the reference
 * (qimpy/dft/electrons/_wavefunction.py:264-275); outputs always have zero padding.
 */
#ifndef QIMPY_GB300_H
#define QIMPY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QGB_ABI_VERSION 2

enum qgb_dtype { QGB_F64 = 0, QGB_F32 = 1 };

enum qgb_status {
  QGB_OK = 0,
  QGB_ERR_INVALID = 1,     /* bad argument: null pointer, size, unsupported grid */
  QGB_ERR_WORKSPACE = 2,   /* workspace smaller than qgb_*_workspace_bytes() */
  QGB_ERR_CUDA = 3,        /* CUDA runtime or launch error */
  QGB_ERR_CUBLAS = 4,      /* cuBLAS error */
  QGB_ERR_UNSUPPORTED = 5, /* valid request the library does not implement */
  QGB_ERR_CUSOLVER = 6     /* cuSOLVER error */
};

/* Flags of qgb_apply_potential. */
#define QGB_ADD_KE 1u       /* out = KE*C + V*C instead of V*C */
#define QGB_ACCUMULATE 2u   /* out += ... instead of out = ... */

/*
 * G-sphere layout of one basis (all k-points of a cell) on the FFT grid
 * N0 x N1 x N2 (N2 fastest).  Built once per basis by the host from the
 * reference's fft_index (qimpy/dft/electrons/_basis.py:186-193): in-sphere
 * points are sorted by linear grid index, so the points with the same first
 * grid index i0 (one "slab") are contiguous in the basis.
 *
 *   n[nk]                       in-sphere count per k
 *   n_slabs[nk]                 number of distinct i0 values touched per k
 *   slab_start[nk][max_slabs+1] basis offset of each slab (last = n[k])
 *   slab_i0[nk][max_slabs]      i0 of each slab
 *   yz[nk][n_tot]               packed (i1 << 16) | i2 of each in-sphere point
 *   row_start[nk][max_slabs+1]  offsets into `rows` of each slab's active i1 list
 *   rows[...]                   distinct i1 values of each slab (z-FFT pencils)
 *   twiddle_{f64,f32}           per axis a, L1[a]*L2[a] complex values
 *                               exp(+2 pi i n1 k2 / N_a), n1 < L1[a], k2 < L2[a],
 *                               axis 0 first; offsets tw_off[a]
 *   ke                          [nk][n_tot] kinetic energy, 0.5 |k+G|^2 (real,
 *                               of the call's dtype)
 *   V                           [N0][N1][N2] real potential in the digit-permuted
 *                               real-space order of qgb_permute_real_space()
 */
typedef struct qgb_sphere {
  int32_t nk, n_tot;
  int32_t N[3];
  int32_t L1[3], L2[3];     /* N[a] = L1[a] * L2[a]; both in {1..10,12,14,15,16} */
  int32_t max_slabs, max_rows;
  int32_t tw_off[3];
  const int32_t* n;
  const int32_t* n_slabs;
  const int32_t* slab_start;
  const int32_t* slab_i0;
  const int32_t* yz;
  const int32_t* row_start;
  const int32_t* rows;
  const void* twiddle;      /* complex of the call's dtype */
  const void* ke;           /* real of the call's dtype */
  const void* V;            /* real of the call's dtype, permuted order */
} qgb_sphere;

/*
 * One unit of a batched local-potential apply: a block of bands of one
 * independent problem (its own cell, grid, k-points and basis).
 *   sphere  DEVICE pointer to a copy of the problem's qgb_sphere
 *   C, out  [nk][nb][n_tot] of that sphere (out may alias C)
 *   planes  >= qgb_potential_workspace_bytes(sphere, nb, dtype) bytes, not
 *           shared with any other item of the batch
 */
typedef struct qgb_batch_item {
  const struct qgb_sphere* sphere;
  const void* C;
  void* out;
  void* planes;
  int32_t nb;
  uint32_t flags;
} qgb_batch_item;

/* Library identification. */
int qgb_abi_version(void);
const char* qgb_last_error(void);

/*
 * Workspace (bytes) that qgb_apply_potential / qgb_hamiltonian need for `nb`
 * bands; any size >= 1 slab-plane per band chunk works, larger sizes let more
 * bands run per launch.  Host function, no device access.
 */
size_t qgb_potential_workspace_bytes(const qgb_sphere* s, int nb, int dtype);

/*
 * Real-space permutation used for V: position p along axis a holds real-space
 * index perm[a][p] = (p / L1) + L2 * (p % L1).  Host function; writes N[a]
 * entries per axis into host array perm (axis 0, then 1, then 2).
 */
int qgb_permute_real_space(const qgb_sphere* s, int32_t* perm);

/*
 * out[k][b] = KE[k] * C[k][b]  (replaces Basis.apply_ke,
 * qimpy/dft/electrons/_basis_ops.py:29-36).
 */
int qgb_apply_ke(const qgb_sphere* s, int dtype, const void* C, void* out, int nb, void* stream);

/*
 * out = gather(FFT(V * IFFT(scatter(C)))) for nb bands at every k of the sphere
 * (replaces Basis.apply_potential for one spin channel,
 * qimpy/dft/electrons/_basis_ops.py:39-113 with _ApplyPotentialKernel 166-204):
 * inverse FFT unnormalised, forward FFT scaled by 1/(N0 N1 N2), padding zeroed.
 * flags: QGB_ADD_KE adds KE*C (fusing Basis.apply_ke), QGB_ACCUMULATE adds into out.
 * `workspace` holds intermediate slab planes (qgb_potential_workspace_bytes).
 */
int qgb_apply_potential(const qgb_sphere* s, int dtype, const void* C, void* out, int nb,
                        unsigned flags, void* workspace, size_t workspace_bytes, void* stream);

/*
 * qgb_apply_potential without a workspace argument, for callers that cannot
 * allocate device memory: host codes whose device memory belongs to an outer
 * framework that forbids allocations by plugins, or code running where
 * cudaMalloc is not allowed (inside a stream capture, or a serving loop with a
 * fixed memory budget).  No counterpart in the reference.
 *
 * Same arguments, flags and results as qgb_apply_potential; the slab-plane
 * scratch is a fixed file-scope device array of qgb_static_scratch_bytes()
 * (32 MiB) that every GPU loading the library holds until exit.  Bands are
 * processed in as many chunks as that scratch needs; a sphere for which even
 * one band does not fit is rejected with QGB_ERR_WORKSPACE.  The function
 * calls no allocator.
 *   - The first call on a device looks up the array's device address (once per
 *     device, with that device current); make that first call before any
 *     stream capture.  A device reset (cudaDeviceReset) gives the device a
 *     new context and the array a new address: the first call after it looks
 *     the address up again, so it too belongs before any capture.
 *   - All calls share the one array and it keeps the previous call's contents;
 *     nothing in it needs to start at zero (every plane is written before it is
 *     read within a call).  Calls that overlap on the GPU (different streams,
 *     or host threads without ordering) race on the array: serialise them.
 */
int qgb_apply_potential_static(const qgb_sphere* s, int dtype, const void* C, void* out, int nb,
                               unsigned flags, void* stream);
size_t qgb_static_scratch_bytes(void);

/*
 * Electron density of a band block: rho[N0][N1][N2] (FP64, natural real-space
 * order) = sum_{k,b} prefac[k][b] |psi_kb(r)|^2 with psi = the unnormalised
 * inverse FFT of the sphere-scattered C (complex128 or complex64 by dtype);
 * prefac [nk][nb] FP64 = f * w_sk / Omega.  rho is zeroed first unless flags
 * has QGB_ACCUMULATE.  Workspace as qgb_apply_potential (band chunks).
 * Replaces Basis.collect_density (qimpy/dft/electrons/_basis_ops.py:207-296,
 * one spin, no spinors) with accum_norm_ (qimpy/math/_linalg.py:31-58).
 */
int qgb_collect_density(const qgb_sphere* s, int dtype, const void* C, int nb, const double* prefac, double* rho,
                        unsigned flags, void* workspace, size_t workspace_bytes, void* stream);

/*
 * Shared memory per CTA the local-potential kernels need for a sphere (host):
 * the largest over the three kernels (the x-phase kernel's), and that of the
 * two y/z-phase kernels alone.
 */
size_t qgb_sphere_smem_bytes(const qgb_sphere* s, int dtype);
size_t qgb_sphere_smem_bytes_yz(const qgb_sphere* s, int dtype);

/*
 * Batched Basis.apply_potential (qimpy/dft/electrons/_basis_ops.py:39-113) for
 * many independent problems with uneven grids and bases: three launches (one
 * per transform phase) for the whole batch.  `items` (device) lists the
 * problems' band blocks; `slab_starts` and `row_starts` (device, n_items + 1
 * prefix sums) give each item's work units: nk * nb * max_slabs for the y/z
 * phases and nk * nb * N1 for the x phase; `slab_item` / `row_item` (device,
 * one int per unit) name the item of every unit; smem_yz / smem_x = max over
 * items of qgb_sphere_smem_bytes_yz / qgb_sphere_smem_bytes.  Launch-only
 * (capturable in a CUDA graph).
 */
int qgb_apply_potential_batched(const qgb_batch_item* items, int n_items, const int* slab_item,
                                const long long* slab_starts, const int* row_item, const long long* row_starts,
                                long long n_slab_units, long long n_row_units, int dtype, size_t smem_yz,
                                size_t smem_x, void* stream);

/*
 * projT[k][b][p] = sum_g conj(beta[k][p][g]) C[k][b][g]  (replaces Wavefunction.proj
 * = beta ^ C, qimpy/dft/electrons/_wavefunction.py:106-123 and
 * _wavefunction_dot.py:18-107).  The sum over the basis is split across CTAs;
 * `workspace` holds the partial sums (qgb_project_workspace_bytes, may be 0),
 * added in a fixed order, so results are reproducible bit for bit.
 */
size_t qgb_project_workspace_bytes(int dtype, int nk, int P, int nb, int n_tot);
int qgb_project(int dtype, const void* beta, const void* C, void* projT, int nk, int P, int nb,
                int n_tot, void* workspace, size_t workspace_bytes, void* stream);

/*
 * Overlaps of two band blocks at every k: out[k][i][j] = sum_g conj(X[k][i][g])
 * Y[k][j][g] for X [nk][nx][n_tot], Y [nk][ny][n_tot] of `dtype`; out is
 * complex128 [nk][nx][ny] for both dtypes (FP32 inputs: FP32 partial sums,
 * added in FP64).  Replaces Wavefunction.dot / ^ for one spin and no spinors
 * (qimpy/dft/electrons/_wavefunction_dot.py:18-107).  Workspace of
 * qgb_dot_workspace_bytes (split-K partials, fixed summation order).
 */
size_t qgb_dot_workspace_bytes(int dtype, int nk, int nx, int ny, int n_tot);
int qgb_dot(int dtype, const void* X, int nx, const void* Y, int ny, int nk, int n_tot, void* out,
            void* workspace, size_t workspace_bytes, void* stream);
/*
 * qgb_dot of complex64 X, Y on the tcgen05 tensor cores (mixed form: the
 * subspace overlaps of Wavefunction.dot, qimpy/dft/electrons/_wavefunction_dot.py:18-107,
 * as split-BF16x3 GEMMs with FP32 accumulation, the basis-range partial sums
 * added in FP64): out complex128 [nk][nx][ny], about 16 significant bits per
 * product.  Workspace of qgb_dot_tc_workspace_bytes; dev_error as for
 * qgb_apply_nonlocal_tc.
 */
size_t qgb_dot_tc_workspace_bytes(int nk, int nx, int ny, int n_tot);
int qgb_dot_tc(const void* X, int nx, const void* Y, int ny, int nk, int n_tot, void* out, void* workspace,
               size_t workspace_bytes, int* dev_error, void* stream);

/*
 * qgb_matmul of complex64 C and M on the tcgen05 tensor cores (mixed form:
 * Wavefunction.matmul, qimpy/dft/electrons/_wavefunction_dot.py:137-191, as
 * one split-BF16x3 GEMM with FP32 accumulation into out): out complex64
 * [nk][n_out][n_tot] (+= with QGB_ACCUMULATE), M complex64 [nk][n_in][n_out];
 * out must not alias C.  Workspace of qgb_matmul_tc_workspace_bytes.
 */
size_t qgb_matmul_tc_workspace_bytes(int nk, int n_in, int n_out, int n_tot);
int qgb_matmul_tc(const void* C, int n_in, int nk, int n_tot, const void* M, int n_out, void* out, unsigned flags,
                  void* workspace, size_t workspace_bytes, int* dev_error, void* stream);

/*
 * The overlap of real (Gamma-point) wavefunctions on the half basis:
 * out[i][j] = Re sum_g w_g conj(X[i][g]) Y[j][g] (imaginary part 0), weight
 * FP64 [n_tot], workspace of qgb_dot_workspace_bytes with nk = 1 (the
 * real-basis branch of qimpy/dft/electrons/_wavefunction_dot.py:55-88).
 */
int qgb_dot_real(int dtype, const void* X, int nx, const void* Y, int ny, int n_tot, const double* weight,
                 void* out, void* workspace, size_t workspace_bytes, void* stream);

/*
 * Band rotation out[k][j][g] = sum_i M[k][i][j] C[k][i][g] (+= with
 * QGB_ACCUMULATE) for C [nk][n_in][n_tot], M [nk][n_in][n_out] and out
 * [nk][n_out][n_tot], all of `dtype`; out must not alias C.  Replaces
 * Wavefunction.matmul / @ (qimpy/dft/electrons/_wavefunction_dot.py:137-191).
 */
int qgb_matmul(int dtype, const void* C, int n_in, int nk, int n_tot, const void* M, int n_out, void* out,
               unsigned flags, void* stream);

/*
 * out[k][b][g] += sum_p beta[k][p][g] (D_all projT[k][b])[p]  (replaces
 * beta @ (D_all @ C.proj), qimpy/dft/electrons/_hamiltonian.py:22-24 with
 * Wavefunction.matmul, _wavefunction_dot.py:137-191).  D is given per atom
 * block (n_atoms blocks of pa x pa).  `work` holds nk*nb*P complex values.
 */
int qgb_apply_nonlocal(int dtype, const void* beta, const void* D, int n_atoms, int pa,
                       const void* projT, void* out, int nk, int nb, int n_tot, void* work,
                       void* stream);

/*
 * HC = KE C + V C + beta D <beta|C>  (replaces Electrons.hamiltonian,
 * qimpy/dft/electrons/_hamiltonian.py:7-29, for a fixed local potential).
 * projT receives <beta|C> (the reference caches it as C.proj).  Workspace of
 * qgb_hamiltonian_workspace_bytes: the slab planes, D <beta|C> and the
 * projection's partial sums.  beta may be NULL when P == 0.
 */
int qgb_hamiltonian(const qgb_sphere* s, int dtype, const void* C, void* HC, int nb,
                    const void* beta, const void* D, int n_atoms, int pa, void* projT,
                    void* workspace, size_t workspace_bytes, void* stream);

size_t qgb_hamiltonian_workspace_bytes(const qgb_sphere* s, int nb, int P, int dtype);

/*
 * Band-wise passes of the Davidson iteration (one read of the bands each; FP64
 * sums; C and HC of `dtype`, [nk][nb_all][n_tot], the pass covers bands
 * [b0, b0 + nb); ke FP64 [nk][n_tot]; per-band results FP64 [nk][nb]):
 *
 * qgb_band_norm_ke: norm = ||C_b||, band_ke = sum_g |C_bg|^2 KE_g (either may be
 *   NULL; ke may be NULL without band_ke); with `weight` (FP64 [n_tot], may be
 *   NULL) every |C_bg|^2 is weighted by w_g (real wavefunctions: 1 on the
 *   Gz = 0 plane, 2 elsewhere).  Replaces Wavefunction.band_norm and band_ke
 *   (qimpy/dft/electrons/_wavefunction.py:226-247).
 * qgb_residual: R = HC_b - eig[k][b0 + b] C_b (eig FP64 [nk][eig_ld]); with
 *   KEref (FP64 [nk][nb]) preconditioned as R / (x + exp(-x)), x = KE / KEref_b;
 *   stored to out [nk][nb][n_tot] (may be NULL) and reduced to norm (may be
 *   NULL, weighted like qgb_band_norm_ke).  Replaces the residual and Davidson.precondition
 *   (qimpy/dft/electrons/_davidson.py:92-99, 177-180).
 * qgb_normalize_bands: X [nk][nb][n_tot] in place: bands with norm < norm_cut
 *   are re-randomised with the reference's seeded generator (state (1 + seed)
 *   + g + n_max (b + nb k), one discarded draw, Box-Muller, damped by
 *   1 / (1 + (4/3 KE)^6), inside the sphere n[k]) and their norm set to 1; the
 *   others are divided by their norm; padding zeroed.  Replaces
 *   Davidson._regularize with Wavefunction.randomize_selected and the
 *   normalisation and constrain that follow (_davidson.py:101-115, 181-183;
 *   _wavefunction_init.py:127-188; _wavefunction.py:264-275).  n: int32 [nk].
 */
int qgb_band_norm_ke(int dtype, const void* C, int nb_all, int b0, int nb, int nk, int n_tot, const double* ke,
                     const double* weight, double* norm, double* band_ke, void* stream);
int qgb_residual(int dtype, const void* HC, const void* C, int nb_all, int b0, int nb, int nk, int n_tot,
                 const double* eig, int eig_ld, const double* ke, const double* KEref, const double* weight,
                 void* out, double* norm, void* stream);
int qgb_normalize_bands(int dtype, void* X, int nb, int nk, int n_tot, const int32_t* n, double* norm,
                        double norm_cut, long long seed, long long n_max, const double* ke, void* stream);

/*
 * Real (Gamma-point) wavefunctions: coefficients on the half-sphere basis
 * Gz >= 0 of the reference's real-wavefunction mode
 * (qimpy/dft/electrons/_basis_real.py:10-106; H-mesh basis, _basis.py:168),
 * rows [nb][n_tot_half], with c(-G) = conj(c(G)) implied.  The local potential
 * runs on the full Gamma sphere (a qgb_sphere with nk = 1 and the potential
 * installed) with two real bands per complex transform.
 *   pack[n_full][2]      per full-sphere entry G: (half index of G, -1) for
 *                        Gz > 0; (half index of -G | bit 31 (conjugate), -1)
 *                        for Gz < 0; (half index of G, half index of -G) on
 *                        the Gz = 0 plane, whose Hermitian part is used
 *   unpack[n_half][2]    full-sphere index of G and of -G of every half entry
 *   plane[n_plane][2]    half index of each Gz = 0 entry and of its -G partner
 *   ke[n_tot_half]       0.5 |G|^2, real of the call's dtype
 *   weight[n_tot_half]   FP64 overlap weight: 1 on Gz = 0, 2 elsewhere, 0 on padding
 */
typedef struct qgb_real_map {
  int32_t n_half, n_tot_half;  /* half-basis entries, padded row length */
  int32_t n_full, n_tot_full;  /* full-sphere entries, its padded row length (the sphere's n_tot) */
  int32_t n_plane;             /* half entries with Gz = 0 */
  const int32_t* pack;
  const int32_t* unpack;
  const int32_t* plane;
  const void* ke;
  const double* weight;
} qgb_real_map;

/*
 * HC = KE C + V C + beta D <beta|C> for real wavefunctions (replaces
 * Electrons.hamiltonian, qimpy/dft/electrons/_hamiltonian.py:7-29, in the
 * reference's real-wavefunction mode): the local potential of ceil(nb / 2)
 * packed full-sphere rows, then <beta|C> = Re sum_G w_G conj(beta) C (projT
 * [nb][P], imaginary parts zero; _wavefunction_dot.py:55-88) and the
 * back-projection.  C, HC [nb][n_tot_half] of `dtype` (must not alias);
 * beta [P][n_tot_half]; D per-atom blocks [n_atoms][pa][pa].  The Gz = 0 plane
 * of the local term is Hermitian.  Workspace of
 * qgb_hamiltonian_real_workspace_bytes.
 */
size_t qgb_hamiltonian_real_workspace_bytes(const qgb_sphere* full, const qgb_real_map* map, int nb, int P,
                                            int dtype);
int qgb_hamiltonian_real(const qgb_sphere* full, const qgb_real_map* map, int dtype, const void* C, void* HC,
                         int nb, const void* beta, const void* D, int n_atoms, int pa, void* projT, void* workspace,
                         size_t workspace_bytes, void* stream);

/*
 * The same in the mixed form (complex64, FP32 local potential): the weighted
 * real projection and the back-projection as tcgen05 split-BF16x3 GEMMs on
 * qgb_beta_split operands of beta [1][P][n_tot_half] (the mixed counterpart
 * of qgb_hamiltonian_real, as qgb_hamiltonian_mixed is of qgb_hamiltonian).
 * dev_error as for qgb_apply_nonlocal_tc.
 */
size_t qgb_hamiltonian_real_mixed_workspace_bytes(const qgb_sphere* full, const qgb_real_map* map, int nb, int P);
int qgb_hamiltonian_real_mixed(const qgb_sphere* full, const qgb_real_map* map, const void* C, void* HC, int nb,
                               const void* beta_split, const void* D, int n_atoms, int pa, void* projT,
                               void* workspace, size_t workspace_bytes, int* dev_error, void* stream);

/*
 * X [nb][n_tot_half] in place: c(G) = (c(G) + conj(c(-G))) / 2 on the Gz = 0
 * plane (replaces BasisReal.symmetrize, qimpy/dft/electrons/_basis_real.py:68-106).
 */
int qgb_symmetrize_real(int dtype, const qgb_real_map* map, void* X, int nb, void* stream);

/*
 * Projectors generated on the device (replaces Ions.get_projectors,
 * qimpy/dft/ions/_ions_projectors.py:14-72):
 *   beta[k][a pa + j][g] = i^l S_lm(q) R_s(|q|) exp(-2 pi i (iG + k).tau_a) / sqrt(volume),
 *   q = (iG + k) Gbasis^T,
 * for atoms a (fractional positions [n_atoms][3], FP64, device) and the atom
 * template of `shells` (host array; projector j runs over the shells in order
 * and, within a shell, over the 2l + 1 real solid harmonics S_lm = |q|^l Y_lm,
 * m = -l..l, l = 1 as (y, z, x); pa = sum (2l + 1)).  Radial R_s:
 *   QGB_RADIAL_GAUSSIAN  (-1)^l (2 pi)^{3/2} sigma^{2l+3} exp(-sigma^2 |q|^2 / 2), the
 *                        transform of r^l Y_lm exp(-r^2 / (2 sigma^2))
 *   QGB_RADIAL_BLIP      quintic blip spline with coefficients coeff[n_coeff]
 *                        (FP64, device) on spacing dq, evaluated as the
 *                        reference's Interpolator (qimpy/math/quintic_spline.py:57-130)
 * iG int32 [nk][n_tot][3], k FP64 [nk][3] and n int32 [nk] on the device;
 * Gbasis FP64 [3][3] row-major on the host.  beta [nk][n_atoms pa][n_tot] of
 * `dtype` (computed in FP64); entries g >= n[k] are zero.  l <= 2, at most 8 shells.
 */
enum qgb_radial_kind { QGB_RADIAL_GAUSSIAN = 0, QGB_RADIAL_BLIP = 1 };
typedef struct qgb_projector_shell {
  int32_t l;
  int32_t kind;         /* enum qgb_radial_kind */
  double sigma;         /* QGB_RADIAL_GAUSSIAN: width (bohr) */
  const double* coeff;  /* QGB_RADIAL_BLIP: blip coefficients (device) */
  int32_t n_coeff;
  double dq;            /* QGB_RADIAL_BLIP: |q| spacing of the coefficients */
} qgb_projector_shell;
int qgb_make_projectors(int dtype, int nk, int n_tot, const int32_t* n, const int32_t* iG, const double* k,
                        const double* Gbasis, int n_atoms, const double* positions, int n_shells,
                        const qgb_projector_shell* shells, double volume, void* beta, void* stream);

/*
 * Mixed-precision nonlocal term on the tcgen05 tensor cores (split-BF16x3,
 * FP32 accumulation):  projT = <beta|C>  and  HC += beta (D projT), complex64
 * (replaces C.proj and beta @ (D_all @ C.proj),
 * qimpy/dft/electrons/_wavefunction.py:106-123 and _hamiltonian.py:22-24).
 *   qgb_beta_split      once per basis: beta complex64 [nk][P][n_tot] -> bf16
 *                       hi/lo operands in `out` (qgb_beta_split_bytes).
 *   qgb_apply_nonlocal_tc  per call; D complex64 per-atom blocks; `workspace`
 *                       of qgb_nonlocal_tc_workspace_bytes; `dev_error` is a
 *                       device int that a kernel sets nonzero (and keeps) if a
 *                       bounded pipeline wait timed out.
 */
size_t qgb_beta_split_bytes(int nk, int P, int n_tot);
int qgb_beta_split(const void* beta, int nk, int P, int n_tot, void* out, size_t out_bytes, void* stream);
size_t qgb_nonlocal_tc_workspace_bytes(int nk, int P, int nb, int n_tot);
int qgb_apply_nonlocal_tc(const void* beta_split, const void* D, int n_atoms, int pa, const void* C, void* HC,
                          void* projT, int nk, int nb, int n_tot, void* workspace, size_t workspace_bytes,
                          int* dev_error, void* stream);
/*
 * The same in two phases, so that the part that reads only C can run beside
 * the local potential (another stream): phases = 1 computes projT and the
 * back-projection operand in `workspace` (HC untouched), phases = 2 then does
 * HC += beta (D projT) from that workspace, phases = 3 both.  Adding 4 to a
 * phases value that includes 2 stores HC = beta (D projT) instead of adding
 * (every entry of HC, padding included, is written).  Between a phase-1 and
 * its phase-2 call the workspace must not be reused.
 */
int qgb_apply_nonlocal_tc_phase(const void* beta_split, const void* D, int n_atoms, int pa, const void* C,
                                void* HC, void* projT, int nk, int nb, int n_tot, void* workspace,
                                size_t workspace_bytes, int* dev_error, int phases, void* stream);

/*
 * Mixed-precision H C (complex64): FP32 KE + local potential (as
 * qgb_apply_potential with QGB_ADD_KE) plus the tensor-core nonlocal term
 * (qgb_apply_nonlocal_tc); replaces Electrons.hamiltonian,
 * qimpy/dft/electrons/_hamiltonian.py:7-29, in the mixed form.  The nonlocal
 * term runs on a library side stream (forked from and joined back to `stream`
 * by events, so the call can be captured) and is stored into HC while the
 * local potential's transforms run; the local potential's last kernel then
 * adds KE C + V C.  beta_split comes from qgb_beta_split; workspace of
 * qgb_hamiltonian_mixed_workspace_bytes.
 */
size_t qgb_hamiltonian_mixed_workspace_bytes(const qgb_sphere* s, int nb, int P);
int qgb_hamiltonian_mixed(const qgb_sphere* s, const void* C, void* HC, int nb, const void* beta_split,
                          const void* D, int n_atoms, int pa, void* projT, void* workspace, size_t workspace_bytes,
                          int* dev_error, void* stream);

/*
 * FP64 eigenpairs of nk Hermitian n x n matrices A ([nk][n][n] complex128,
 * row-major) in one batched cuSOLVER call on `stream`: W [nk][n] ascending
 * eigenvalues; A is overwritten with V^H (row j = conj of eigenvector j);
 * info [nk] device ints, nonzero where a matrix failed to converge.
 * Workspace of qgb_subspace_eigh_workspace_bytes(nk, n) (0 = query failed).
 * Replaces the torch.linalg.eigh of the Davidson subspace problems
 * (qimpy/dft/electrons/_davidson.py:164-168; qimpy/math/_linalg.py:143-183).
 */
size_t qgb_subspace_eigh_workspace_bytes(int64_t nk, int64_t n);
int qgb_subspace_eigh(void* A, double* W, int* info, int64_t nk, int64_t n, void* workspace,
                      size_t workspace_bytes, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* QIMPY_GB300_H */
