/*
 * pychem_gb300 -- C ABI of the GB300 (sm_103a) Hartree-Fock integral and SCF library.
 *
 * Two layers, both plain C (pointers, sizes, an opaque CUDA stream handle):
 *
 *  1. Drop-in layer for the upstream `_c_ints` CPython extension
 *     (Methods/_c_ints.c:68-81).  One function per upstream method, same argument
 *     order and meaning; arrays are HOST buffers laid out exactly as the upstream
 *     NumPy arrays (C-contiguous float64), outputs are written in place (the contract
 *     functions accumulate, as upstream).  Each call copies to the GPU, runs one
 *     kernel, copies back and synchronises.  Return value: 0 on success, otherwise a
 *     PCG_ERR_* code with a message from pcg_last_error().
 *
 *  2. Batched whole-molecule layer used by the GPU SCF: DEVICE pointers, caller-owned
 *     buffers, an explicit stream, asynchronous.  Replaces the per-quartet Python loops
 *     of Methods/hartree_fock.py:207-355 (core matrices, Schwarz pass, screened ERI
 *     store, J/K contraction).
 */
#ifndef PYCHEM_GB300_H
#define PYCHEM_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PCG_OK 0
#define PCG_ERR_CUDA 1
#define PCG_ERR_ARG 2
#define PCG_ERR_UNSUPPORTED 3
#define PCG_ERR_NOTINIT 4
#define PCG_ERR_CAPACITY 5

/* ---------------------------------------------------------------------------------
 * Library
 * --------------------------------------------------------------------------------- */
int pcg_version(void);
const char *pcg_last_error(void);
/* Build the Boys-function table on the current device (idempotent). */
int pcg_device_init(void);

/* ---------------------------------------------------------------------------------
 * 1. Drop-in layer: the 11 methods of the upstream `_c_ints` module.
 *    Shapes below use ncart(l) = (l+1)(l+2)/2; "[r][c]" means r*c doubles row-major.
 * --------------------------------------------------------------------------------- */

/* Methods/_c_ints.c:114-154 (c_ints/shellpair_quantities.c:5-38).
 * sigmas, overlaps [n_alpha][n_beta]; centres [n_alpha][n_beta][3]. */
int pcg_shellpair_quantities(double *sigmas, double *overlaps, double *centres,
                             const double *alpha_exps, const double *A, int n_alpha,
                             const double *beta_exps, const double *B, int n_beta);

/* Methods/_c_ints.c:158-191 (c_ints/two_electron_bound.c:5-27).
 * bounds [nla*nlb*nlc*nld]; C_P [nla][nlb]; C_Q [nlc][nld]. */
int pcg_two_electron_bound(double *bounds, const double *C_P, const double *C_Q,
                           int nla, int nlb, int nlc, int nld);

/* Methods/_c_ints.c:195-245 (c_ints/two_electron_fundamentals.c:6-95; with
 * ints_type 1 c_ints/two_electron_scattering.c:6-81, the j0(S r12) operator at
 * S = grid_value >= 0, z^-m j_m(z) by the regimes of spherical_bessel_j.c).
 * fundamentals [m+1][na*nb][nc*nd]; sigma/U [na][nb], [nc][nd]; P [na][nb][3];
 * Q [nc][nd][3]; R [na*nb][nc*nd][3] (output). */
int pcg_two_electron_fundamentals(double *fundamentals, const double *sigma_P, const double *U_P,
                                  const double *P, const double *sigma_Q, const double *U_Q,
                                  const double *Q, double *R, int na, int nb, int nc, int nd,
                                  int m, int ints_type, double grid_value);

/* Methods/_c_ints.c:249-301 (c_ints/two_electron_vrr.c:4-141).
 * target [ncart(lbra)*na*nb][ncart(lket)*nc*nd]; base0/base1 [ncart(lbra-1)*na*nb][..];
 * base2/base3 [ncart(lbra-2)*na*nb][..] (read when lbra >= 2); base4
 * [ncart(lbra-1)*na*nb][ncart(lket-1)*nc*nd] (read when lket >= 1); zeta [na][nb];
 * eta [nc][nd]; kappa [na] (kappa_index 0) or [nb]; Rx [3]; R [na*nb][nc*nd][3]. */
int pcg_two_electron_vrr(double *target, const double *base0, const double *base1,
                         const double *base2, const double *base3, const double *base4,
                         const double *zeta, const double *eta, const double *kappa,
                         const double *Rx, const double *R, int na, int nb, int nc, int nd,
                         int lbra, int lket, int kappa_index);

/* Methods/_c_ints.c:305-344 (c_ints/two_electron_contract.c:3-57); accumulates.
 * contracted [ncart(lbra)][ncart(lket)]; primitive [ncart(lbra)*na*nb][ncart(lket)*nc*nd]. */
int pcg_two_electron_contract(double *contracted, const double *primitive, const double *cc_bra,
                              const double *cc_ket, int na, int nb, int nc, int nd, int lbra,
                              int lket);

/* Methods/_c_ints.c:348-385 (c_ints/two_electron_hrr.c:4-94).
 * goofy 0: target [ncart(la)*ncart(lb+1)][ncart(lc)*ncart(ld)], base0 (la+1, lb),
 * base1 (la, lb); goofy 1: target [ncart(la+1)*ncart(lb)][..], base0 (la, lb+1),
 * base1 (la, lb), rows of base0 indexed with the upstream stride. */
int pcg_two_electron_hrr(double *target, const double *base0, const double *base1,
                         const double *Rx, int la, int lb, int lc, int ld, int goofy);

/* Methods/_c_ints.c:389-431 (c_ints/one_electron_fundamentals.c:6-103).
 * fundamentals [m+1][na][nb]; Rc [3]. */
int pcg_one_electron_fundamentals(double *fundamentals, const double *sigma_P, const double *U_P,
                                  const double *P, const double *Rc, double Z, int na, int nb,
                                  int m);

/* Methods/_c_ints.c:435-501 (c_ints/one_electron_vrr.c:4-82); base_list holds n_base
 * pointers.  atom_index -1: overlap (base0 [ncart(la-1)*na][nb], base1
 * [ncart(la-2)*na][nb]); otherwise nuclear attraction (base0, base1 [ncart(la-1)*na][nb],
 * base2, base3 [ncart(la-2)*na][nb]).  target [ncart(la)*na][nb]. */
int pcg_one_electron_vrr(double *target, const double *const *base_list, const double *sigma_P,
                         const double *P, const double *Ra, const double *Rc, int atom_index,
                         int n_base, int na, int nb, int la);

/* Methods/_c_ints.c:505-552 (c_ints/one_electron_hrr.c:4-75).
 * target [ncart(la)*na][ncart(lb)*nb]; base0 (la+1, lb-1); base1 (la, lb-1). */
int pcg_one_electron_hrr(double *target, const double *const *base_list, const double *Rab,
                         int n_base, int na, int nb, int la, int lb);

/* Methods/_c_ints.c:556-605 (c_ints/one_electron_kinetic.c:4-75).
 * target [ncart(la)*na][ncart(lb)*nb]; base0 (la, lb+2), base1 (la, lb), base2 (la, lb-2). */
int pcg_one_electron_kinetic(double *target, const double *const *base_list, const double *exB,
                             int n_base, int na, int nb, int la, int lb);

/* Methods/_c_ints.c:609-644 (c_ints/one_electron_contract.c:3-51); accumulates.
 * target [ncart(la)][ncart(lb)]; base [ncart(la)*na][ncart(lb)*nb]; cc [na][nb]. */
int pcg_one_electron_contract(double *target, const double *base, const double *cc, int na,
                              int nb, int la, int lb);

/* ---------------------------------------------------------------------------------
 * 2. Batched layer (device pointers, asynchronous on `stream`, a cudaStream_t).
 * --------------------------------------------------------------------------------- */

/* Shells of a molecule in upstream AO order (Util/structures.py:464-523).
 * pr_cc: contraction coefficient times (2a)^{(l+1.5)/2} times the normalisation of
 * the pure-axis Cartesian component (Util/structures.py:843,850-856). */
typedef struct {
  int nshell, nprim, natom, nbf;
  const int *sh_l, *sh_nprim, *sh_prim, *sh_ao, *sh_atom;
  const double *sh_xyz, *pr_exp, *pr_cc, *at_xyz, *at_z;
  /* Matrix layout.  One molecule: ld = nbf, sh_blk = sh_at0 = sh_nat = NULL.  An
   * ensemble of molecules in one set of launches: sh_ao holds AO offsets local to the
   * shell's molecule, matrix element (p, q) of that molecule lives at
   * sh_blk[shell] + p * ld + q, and nuclear attraction for the shell runs over atoms
   * [sh_at0[shell], sh_at0[shell] + sh_nat[shell]). */
  int ld;
  const long long *sh_blk;
  const int *sh_at0, *sh_nat;
} pcg_basis_t;

/* Shell pairs (A = higher angular momentum) and their primitive-pair data. */
typedef struct {
  int npair, npp;
  const int *A, *B, *ppoff, *npp_of;
  const double *AB, *zeta, *P, *PA, *K, *oo2z;
  const float *Kf;
  /* Optional (NULL allowed): per pair 4 ints (first AO of A | (A == B) << 30, first AO
   * of B, low and high 32 bits of the molecule block offset), filled by pcg_pair_ao;
   * the Fock digestion reads it instead of the shell tables. */
  const int *ao4;
  /* Optional (NULL allowed): per primitive pair 8 floats (zeta, P-A xyz, 1/(2 zeta), K,
   * 0, 0), filled by pcg_pair_data_f32; the FP32 ERI kernels read it instead of
   * converting the double arrays. */
  const float *pf8;
} pcg_pairs_t;

/* Primitive-pair data for npair pairs (replaces the per-pair ShellPair set-up,
 * Util/structures.py:918-956).  Outputs sized npair*3 (AB) and npp (*3). */
int pcg_pair_data(const pcg_basis_t *basis, int npair, const int *A, const int *B,
                  const int *ppoff, double *AB, double *zeta, double *P, double *PA, double *K,
                  float *Kf, double *oo2z, void *stream);

/* The packed FP32 primitive-pair table pcg_pairs_t.pf8 (npp x 8 floats) from the
 * double arrays of pcg_pair_data. */
int pcg_pair_data_f32(int npp, const double *zeta, const double *PA, const double *oo2z, const float *Kf,
                      float *pf8, void *stream);

/* The per-pair AO table pcg_pairs_t.ao4 (npair x 4 ints) from the shell tables. */
int pcg_pair_ao(const pcg_basis_t *basis, int npair, const int *A, const int *B, int *ao4, void *stream);

/* Overlap S and core Hamiltonian H = T + V, nbf x nbf, all shell pairs listed
 * (Methods/hartree_fock.py:207-224 over Methods/integrals.py:220-370). */
int pcg_one_electron(const pcg_basis_t *basis, int npair, const int *A, const int *B, double *S,
                     double *H, void *stream);

/* ERI class id of (la lb|lc ld), la>=lb, lc>=ld, pair class of bra >= ket; -1 if none. */
int pcg_eri_class_id(int la, int lb, int lc, int ld);
/* spherical elements per quartet of a class */
int pcg_eri_class_nout(int cls);

/* Contracted, normalised spherical blocks of ntask quartets (tasks = ntask int pairs
 * {bra pair, ket pair}) of one class into store[k*ntask + t].  fp32 != 0 computes in
 * single precision (for quartets below the mixed-precision Schwarz threshold). */
int pcg_eri_class(int cls, const pcg_basis_t *basis, const pcg_pairs_t *pairs, const int *tasks,
                  int ntask, double *store, int fp32, void *stream);

/* Schwarz factor Q[pair] = sqrt(max (mn|mn)) from diagonal blocks of a diagonal class. */
int pcg_schwarz_class(int cls, const int *tasks, int ntask, const double *store, double *Q,
                      void *stream);

/* Expand screened quartet rows into task pairs: row r pairs bra pair bra[r] with the
 * kets ket[qstart[r] + q] for q < off[r+1] - off[r] - diag[r], and with itself last
 * when diag[r]; its tasks are written at [off[r], off[r+1]) of out_tasks (int2). */
int pcg_expand_tasks(int nbra, const int *bra, const int *ket, const long long *off,
                     const int *qstart, const int *diag, long long ntask, int *out_tasks,
                     void *stream);

/* Closed-shell Fock digestion: G += contributions of the stored blocks of one class
 * with density D (nbf x nbf); F = H + (G + G^T)/2 via pcg_fock_build. */
int pcg_digest_class(int cls, const pcg_basis_t *basis, const pcg_pairs_t *pairs, const int *tasks,
                     int ntask, const double *store, const double *D, double *G, void *stream);
/* Unrestricted digestion (Methods/hartree_fock.py:329-355 with separate alpha and beta
 * densities): GJ += the Coulomb part of (D_a + D_b)/2, GKa / GKb += the exchange parts
 * of D_a / D_b, so that F_s = H + (G + G^T)/2 with G = GJ + GKs equals
 * H + J[D_a + D_b] - K[D_s]. */
int pcg_digest_class_u(int cls, const pcg_basis_t *basis, const pcg_pairs_t *pairs, const int *tasks,
                       int ntask, const double *store, const double *Da, const double *Db, double *GJ,
                       double *GKa, double *GKb, void *stream);
/* Electron-scattering integrals (ab|j0(S r12)|cd) of one class for a task list, same
 * store layout as pcg_eri_class (FP64): the operator of Methods/properties.py:20-23,
 * fundamentals of Methods/c_ints/two_electron_scattering.c:6-81 with z^-m j_m(z) by
 * the regimes of spherical_bessel_j.c:5-81.  S >= 0 is the momentum transfer in the
 * reference's units (inverse bohr).  Used for the Schwarz pass (diagonal tasks) and
 * the screened store of each grid value. */
int pcg_scattering_class(int cls, const pcg_basis_t *basis, const pcg_pairs_t *pairs, const int *tasks,
                         int ntask, double S, double *store, void *stream);
/* Co-density digestion for non-orthogonal CI (Methods/noci.py:243-300 evaluates
 * hartree_fock.py:345-347 on the non-symmetric co-densities of Lowdin-paired
 * determinants): nd densities W, consecutive nbf x nbf row-major blocks; per density
 * GJ += the Coulomb part of (W + W^T)/2 and GK += both orientations of the exchange
 * blocks, so that J[W] = (GJ + GJ^T)/4 and K[W] = -GK/2 with
 * J_ab = sum_cd (ab|cd) W_cd, K_ad = sum_bc (ab|cd) W_cb.  One molecule (no
 * ensemble block table). */
int pcg_digest_class_co(int cls, const pcg_basis_t *basis, const pcg_pairs_t *pairs, const int *tasks,
                        int ntask, const double *store, int nd, const double *W, double *GJ, double *GK,
                        void *stream);
int pcg_fock_build(int n, const double *H, const double *G, double *F, void *stream);
/* Same for nblocks consecutive ld x ld blocks (an ensemble of molecules). */
int pcg_fock_build_batched(int nblocks, int ld, const double *H, const double *G, double *F, void *stream);

/* No counterpart in the upstream code.  The same Fock build as pcg_digest_class over
 * nclass classes followed by pcg_fock_build, for callers that cannot allocate device
 * memory (their GPU memory belongs to another allocator or to a pool fixed at
 * start-up): the nbf x nbf accumulator lives in a static device array inside the
 * library, so the caller passes only inputs (H, D, per class: class id, task list,
 * task count, store -- host arrays of device pointers) and the output F.
 * Limit: nbf <= 512 (2 MiB held on every GPU that loads the library); larger nbf
 * returns PCG_ERR_CAPACITY.  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress) and should come before any stream capture.  Calls
 * share the array; calls that overlap on the GPU race and must be serialised. */
int pcg_fock_build_noalloc(const pcg_basis_t *basis, const pcg_pairs_t *pairs, int nclass,
                           const int *cls, const int *const *tasks, const int *ntask,
                           const double *const *stores, const double *H, const double *D, double *F,
                           void *stream);

/* Scatter the stored blocks of one class into a dense nbf^4 tensor with the 8-fold
 * symmetry (Methods/hartree_fock.py:314-325). */
int pcg_dense_class(int cls, const pcg_basis_t *basis, const pcg_pairs_t *pairs, const int *tasks,
                    int ntask, const double *store, double *eri, void *stream);

/* The same with the bra pair packed, E[row(a, b)][c][d] with a >= b: the input of the
 * first MP2 quarter transform, which keeps the bra symmetry (Methods/mp2.py:43-69
 * transforms the full tensor).  row(a, b) = pairmap[pair(a, b)], pair(a, b) =
 * a(a+1)/2 + b, so that only the AO pairs some stored quartet contains get rows
 * (pairmap NULL: row = pair(a, b), nbf(nbf+1)/2 rows); E: rows x nbf x nbf doubles. */
int pcg_dense_pairs_class(int cls, const pcg_basis_t *basis, const pcg_pairs_t *pairs, const int *tasks,
                          int ntask, const double *store, const int *pairmap, double *E, void *stream);
/* The symmetric pair matrix of the compact rows: M[pairmap[pair(a, b)]][pairmap[pair(c, d)]]
 * = (ab|cd) (both triangles; rows x rows doubles, zeroed by the caller), for the
 * elements whose bra and ket pairs both have rows; with pcg_unpack_pairs(rows, nbf, rows,
 * pairmap, M, E) it gives the tensor of pcg_dense_pairs_class with half the scattered
 * stores. */
int pcg_sym_pairs_class(int cls, const pcg_basis_t *basis, const pcg_pairs_t *pairs, const int *tasks, int ntask,
                        const double *store, const int *pairmap, long long rows, double *M, void *stream);
/* used[p] = 1 (bytes, zeroed by the caller, one per shell pair) for both shell pairs of
 * every task (x, y) of a class list with x != y: the pairs that some off-diagonal
 * stored quartet contains (the rows of the compact pair tensor). */
int pcg_mark_pairs(const int *tasks, int ntask, unsigned char *used, void *stream);
/* colmap[a*n + b] = pairmap[pair(a, b)] (pairmap NULL: pair(a, b) itself), n x n ints:
 * where each (a, b) sits in a pair-packed row, -1 for nowhere. */
int pcg_pair_colmap(int n, const int *pairmap, int *colmap, void *stream);
/* out[r][a][b] = in[r * len + colmap[a*n + b]] (0 where colmap is -1) for r < R,
 * a, b < n: pair-packed rows of length len unpacked (colmap from pcg_pair_colmap); a
 * row of up to 12,800 doubles is staged in shared memory. */
int pcg_unpack_pairs(long long R, int n, int len, const int *colmap, const double *in, double *out, void *stream);

/* FP64-accurate GEMM with every Ozaki level in one tcgen05 tensor-core kernel (no
 * upstream counterpart; it carries the AO->MO transform of Methods/mp2.py:43-69 and
 * the density C_occ C_occ^T of Methods/hartree_fock.py:179-184):
 *   C[m*sCm + n*sCn] (+)= sum_k X[m*ldx + k] * Y[k*sYk + n*sYn],  0 <= m < M, n < N.
 * X (rows contiguous along k, ldx >= K) is split into nslice 7-bit BF16 digit slices
 * inside the kernel; Y is split once into the workspace.  nslice 6 or 7;
 * K * (nslice + 2) < 4096; workspace: pcg_ozaki_tc_workspace(N, K, nslice) bytes,
 * 256-byte aligned, caller-owned device memory.  pcg_ozaki_tc_status: the error flag
 * a kernel sets when it gives up on a bounded wait (0 = none), read synchronously. */
size_t pcg_ozaki_tc_workspace(int N, int K, int nslice);
int pcg_ozaki_gemm_tc(long long M, int N, int K, const double *X, long long ldx, const double *Y, long long sYk,
                      long long sYn, double *C, long long sCm, long long sCn, int nslice, int accumulate,
                      void *workspace, size_t ws_bytes, void *stream);
int pcg_ozaki_tc_status(const void *workspace, void *stream);

/* Small dense FP64 algebra of the SCF iteration (no upstream counterpart as kernels;
 * they replace the numpy products of Methods/hartree_fock.py:168-184,226-237 and the
 * DIIS of Methods/hf_extensions/diis.py:32-41,108-112).
 * pcg_dgemm: C[b][m][n] = alpha sum_k A[b][m][k] B[b][k][n] + beta C[b][m][n], element
 *   strides for every axis (transposes by strides); beta = 0 does not read C.
 * pcg_oa_correction: E (n x n) of one Ogita-Aishima refinement step X <- X + X E from
 *   S = X^T A X and R = I - X^T X; mode 0 decouples the first nocc columns from the
 *   rest, mode 1 separates every pair with |lam_j - lam_i| > *delta (a device scalar,
 *   NULL = 0); lam (optional, n) receives the Rayleigh quotients
 *   S_ii / (1 - R_ii).
 * pcg_diis_step: store F and residual R (len doubles each) in slot state[0] % cap of
 *   the rings focks / resids (cap x len), add the new row of the residual
 *   inner-product matrix Bm (cap x cap), solve the C1 system over the slots in use
 *   (oldest dropped while singular), write the coefficients (cap) and the
 *   extrapolated Fx (len), and advance state[0].  row: cap doubles of scratch.  No
 *   host round trip. */
int pcg_dgemm(int batch, int M, int N, int K, double alpha, const double *A, long long sAb, long long sAm,
              long long sAk, const double *B, long long sBb, long long sBk, long long sBn, double beta, double *C,
              long long sCb, long long sCm, long long sCn, void *stream);
int pcg_oa_correction(int n, int nocc, int mode, const double *delta, const double *S, const double *R, double *E,
                      double *lam, void *stream);
int pcg_diis_step(long long len, int cap, int *state, const double *F, const double *R, double *focks,
                  double *resids, double *Bm, double *row, double *coef, double *Fx, void *stream);

/* Closed-shell MP2 energy sums (replaces the numpy sums of Methods/mp2.py:71-94): from
 * X(i,a,j,b) = (ia|jb) stored at ((b*o + j)*v + a)*o + i and the orbital energies eo
 * (o), ev (v), part[2p] and part[2p+1] (p = b*o + j, o*v blocks) receive block partials
 * of s1 = sum X^2/D and s2 = sum X(i,a,j,b) X(i,b,j,a)/D, D = e_i + e_j - e_a - e_b.
 * E_MP2 = 2 s1 - s2; same spin s1 - s2, opposite spin s1.  One kernel. */
int pcg_mp2_pair_sums(int o, int v, const double *X, const double *eo, const double *ev, double *part,
                      void *stream);

/* Batched symmetric eigensolver (no upstream counterpart; replaces the LAPACK eigh of
 * Methods/hartree_fock.py:172-175,226): parallel cyclic Jacobi, one CTA per matrix
 * (FP32 above n = 160: a few CTAs, each with a share of V's rows).
 * A: batch x n x n FP64 (read only); w: batch x n eigenvalues (unsorted, matching the
 * columns of V); V: batch x m x m with m = n rounded up to even, FP64 (fp32 = 0,
 * n <= 136) or FP32 (fp32 = 1, n <= 334); V0 (optional, same type/layout as V):
 * starting rotation, i.e. A is diagonalised as V0 * (V0^T A V0-space) -- pass NULL
 * for the identity.  info (optional): sweeps used per matrix. */
int pcg_jacobi_eigh(int batch, int n, const double *A, double *w, void *V, int fp32, const void *V0,
                    int max_sweeps, double tol, int *info, void *stream);

/* Learned initial guess (no upstream counterpart; upstream's guesses are the core
 * Hamiltonian and MO files, Methods/hartree_fock.py:35-57).  Dense-layer kernels:
 * C[m][n] (+)= sum_k A[m*sam + k*sak] B[k*sbk + n*sbn] with FP32 A, FP32 or BF16 B
 * (b_bf16), FP32 accumulation, optional epilogue Z = C + bias, C = silu(Z) (act = 1);
 * G *= silu'(Z); column sums; masked squared error (dY = 2 (Y - T) mask * inv_count,
 * loss += sum of squares * inv_count); Adam on FP32 master weights with an optional
 * BF16 copy (bias-corrected by step). */
int pcg_mlp_gemm(int M, int N, int K, const float *A, long long sam, long long sak, const void *B,
                 int b_bf16, long long sbk, long long sbn, float *C, int ldc, int accumulate,
                 const float *bias, float *Z, int act, void *stream);
int pcg_mlp_dsilu(long long n, float *dY, const float *Z, void *stream);
int pcg_mlp_colsum(int M, int N, const float *G, float *db, void *stream);
int pcg_mlp_mse(long long n, const float *Y, const float *T, const float *mask, float inv_count,
                float *dY, float *loss, void *stream);
int pcg_mlp_adam(long long n, float *w, const float *g, float *m, float *v, void *w_bf16, float lr,
                 float b1, float b2, float eps, int step, void *stream);

/* Arithmetic-throughput probe (measurement support, no upstream counterpart): blocks x
 * threads threads each run 8 independent FMA chains of `iters` steps in FP64 (fp32 = 0)
 * or FP32, writing one value per thread to `out` (blocks*threads elements). */
int pcg_fma_probe(int blocks, int threads, int iters, int fp32, void *out, void *stream);

#ifdef __cplusplus
}
#endif
#endif
