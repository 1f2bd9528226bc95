/*
 * votca_gb300_bse.h -- C ABI of the GB300-native BSE hot path.
 *
 * A drop-in for VOTCA-XTP's matrix-free BSE Hamiltonian product and the
 * Davidson eigensolver that drives it.  Every entry point takes plain
 * pointers and 64-bit sizes, returns an int status (0 = success, see
 * bse_status) and never throws; bse_last_error() returns a thread-local
 * message for the last failure on the calling thread.
 *
 * Conventions (identical to the reference):
 *   - matrices are column-major FP64; sizes are int64 (votca::Index);
 *   - the BSE pair index is I(v, c) = ctotal * v + c, virtual index fastest
 *     (xtp/include/votca/xtp/vc2index.h:42-44);
 *   - the operator applies  cqp*Hqp + cx*Hx - cd*Hd - cd2*Hd2
 *     (BSE_OPERATOR<cqp,cx,cd,cd2>, xtp/include/votca/xtp/bse_operator.h:40-87);
 *   - Mmn is the reference's TCMatrix_gwbse: msize() slices, slice m a
 *     column-major [nsize() x auxsize()] matrix (threecenter.h:70-142).
 *
 * Threading: a handle may be used from one host thread at a time; every call
 * is synchronous on return (host-pointer calls) or stream-ordered on the
 * stream passed in (the *_device calls).
 */
#ifndef VOTCA_GB300_BSE_H
#define VOTCA_GB300_BSE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum bse_status {
  BSE_OK = 0,
  BSE_ERR_ARGUMENT = 1,      /* shape / option error (the reference throws std::runtime_error) */
  BSE_ERR_OUT_OF_MEMORY = 2, /* device allocation failed (CudaMatrix::throw_if_not_enough_memory_in_gpu) */
  BSE_ERR_CUDA = 3,          /* CUDA runtime error */
  BSE_ERR_TIMEOUT = 4,       /* a bounded device wait gave up */
  BSE_ERR_NUMERICAL = 5,     /* small eigenproblem failed, Gram-Schmidt linear dependence, ... */
  BSE_ERR_UNSUPPORTED = 6    /* option not supported by this library */
} bse_status;

typedef enum bse_precision {
  BSE_PRECISION_FP64 = 0,   /* every product in FP64 (the plain drop-in) */
  BSE_PRECISION_MIXED = 1,  /* Hx/Hd/Hd2 contractions as BF16x3 split products on
                               tcgen05 tensor cores with FP32 accumulation;
                               Hqp and all Davidson algebra in FP64 */
  BSE_PRECISION_SLICED = 2  /* Hx/Hd/Hd2 contractions as Ozaki slice products on the
                               tcgen05 tensor cores: each FP64 operand cut into five 7-bit
                               digit planes (power-of-two scale per run of <= 1024 K
                               elements), every pair of digit levels up to the fifth
                               accumulated exactly in FP32 over one run, runs and pairs
                               summed in FP64, intermediates kept in FP64; agrees with the
                               FP64 product to about 1e-11 of its scale */
} bse_precision;

/* BSEOperator_Options, xtp/include/votca/xtp/bse_operator.h:32-38 (absolute MO indices). */
typedef struct bse_options {
  int64_t homo;
  int64_t rpamin;
  int64_t qpmin;
  int64_t vmin;
  int64_t cmax;
} bse_options;

/* Window of a TCMatrix_gwbse (TCMatrix_gwbse::Initialize, threecenter.cc:29-48). */
typedef struct bse_mmn_desc {
  int64_t auxsize; /* Naux */
  int64_t mmin, mmax;
  int64_t nmin, nmax;
} bse_mmn_desc;

typedef struct bse_handle bse_handle;

/*
 * Create a device-resident BSE operator from host data.  Replaces the
 * construction of BSE_OPERATOR(epsilon_0_inv, Mmn, Hqp) + configure(opt)
 * (bse_operator.h:44-48, bse_operator.cc:28-37).  The Mmn blocks the product
 * needs (vv, vc, cv, cc in the BSE window) are staged into HBM once, here,
 * instead of per matvec as the reference's CudaPipeline does
 * (openmp_cuda.cc:299-407).
 *   mmn_slices: msize pointers; slice m is column-major nsize x auxsize
 *               (the data() of Mmn_[m]).
 *   epsilon_0_inv: auxsize screening weights (BSE::epsilon_0_inv_).
 *   hqp: column-major Hqp, leading dimension ldh >= hqp_size, occupied first;
 *        its leading (vtotal+ctotal) window is used as by BSE_OPERATOR::Hqp_row.
 */
int bse_op_create(const bse_mmn_desc *mmn, const double *const *mmn_slices,
                  const double *epsilon_0_inv, const double *hqp, int64_t ldh,
                  int64_t hqp_size, const bse_options *opt, int32_t precision,
                  bse_handle **out);

/* Same, with a dense screening matrix W (auxsize x auxsize, symmetric) in place
 * of the diagonal epsilon_0_inv: Hd = sum_PQ M^P W_PQ M^Q.  W is folded into
 * the vv (and cv) blocks at staging. */
int bse_op_create_dense_screening(const bse_mmn_desc *mmn,
                                  const double *const *mmn_slices,
                                  const double *W, const double *hqp,
                                  int64_t ldh, int64_t hqp_size,
                                  const bse_options *opt, int32_t precision,
                                  bse_handle **out);

/* ---- Unrestricted (UKS) BSE operator ---- */

/* BSEOperatorUKS_Options (xtp/include/votca/xtp/bse_operator_uks.h:31-38). */
typedef struct bse_uks_options {
  int64_t homo_alpha;
  int64_t homo_beta;
  int64_t rpamin;
  int64_t qpmin;
  int64_t vmin;
  int64_t cmax;
} bse_uks_options;

/* Create a device-resident unrestricted BSE operator: replaces the construction of
 * BSE_OPERATOR_UKS(epsilon_0_inv, TCMatrix_gwbse_spin{alpha, beta}, Hqp_alpha, Hqp_beta)
 * + configure(opt) (bse_operator_uks.h:41-55, bse_operator_uks.cc:37-43).  Each spin
 * channel is given as bse_op_create takes one Mmn (slices, window) and its own Hqp
 * (window-local, occupied first); both share epsilon_0_inv (same auxsize).  The operator
 * acts on [x_alpha; x_beta] (alpha pairs first, pair index v * ctotal + c per channel,
 * vtotal = homo - vmin + 1, ctotal = cmax - homo); its size is the sum of the two channels.
 * A channel without occupied (homo = vmin - 1) or virtual (homo = cmax) levels in the window
 * carries an empty block, as the reference's setup_block (bse_operator_uks.cc:25-35): the
 * operator is then the other channel's, without cross-spin terms (both empty: an error).
 * The returned handle serves bse_op_size / bse_op_matmul(_device) / bse_op_diagonal(_device)
 * / bse_ham_matmul / bse_davidson_solve with BSE_OPERATOR_UKS<cqp, cx, cd, cd2>
 * coefficients (ExcitonUKSOperator_TDA = 1,1,1,0; ExcitonUKSOperator_BTDA_B = 0,1,0,1;
 * HdUKSOperator = 0,0,1,0; Hd2UKSOperator = 0,0,0,1; QpUKSOperator = 1,0,0,0;
 * HxUKSOperator = 0,1,0,0, bse_operator_uks.h:111-124).  Products follow
 * BSE_OPERATOR_UKS::matmul (bse_operator_uks.cc:220-270): same-spin Hqp, Hx, Hd, Hd2 per
 * channel, the cross-spin TDA term -cd sum_P w_P M_s(c1, v1, P) M_s'(v2, c2, P) and the
 * cross-spin -cd2 Hd2 term; the diagonal has the same-spin terms only (:283-352).
 * precision: BSE_PRECISION_MIXED applies to the same-spin blocks; the cross-spin products
 * run in FP64.  Not supported for UKS handles: bse_op_matmul_device_noalloc,
 * bse_op_eig_gradient, bse_op_profile, lockstep batches (BSE_ERR_ARGUMENT). */
int bse_uks_op_create(const bse_mmn_desc *mmn_alpha, const double *const *mmn_alpha_slices,
                      const bse_mmn_desc *mmn_beta, const double *const *mmn_beta_slices,
                      const double *epsilon_0_inv, const double *hqp_alpha, int64_t ldh_alpha,
                      int64_t hqp_alpha_size, const double *hqp_beta, int64_t ldh_beta,
                      int64_t hqp_beta_size, const bse_uks_options *opt, int32_t precision,
                      bse_handle **out);

/* Same, with a dense symmetric screening matrix W (auxsize x auxsize) in place of the diagonal
 * epsilon_0_inv: every direct term uses sum_PQ M^P W_PQ M^Q.  With W = U diag(w) U^T this is the
 * operator BSE_UKS::SetupDirectInteractionOperator builds by rotating both Mmn with the
 * eigenvectors U of eps and screening with w (bse_uks.cc:135-157). */
int bse_uks_op_create_dense_screening(const bse_mmn_desc *mmn_alpha, const double *const *mmn_alpha_slices,
                                      const bse_mmn_desc *mmn_beta, const double *const *mmn_beta_slices,
                                      const double *W, const double *hqp_alpha, int64_t ldh_alpha,
                                      int64_t hqp_alpha_size, const double *hqp_beta, int64_t ldh_beta,
                                      int64_t hqp_beta_size, const bse_uks_options *opt, int32_t precision,
                                      bse_handle **out);

/* ---- Screening that feeds Hd (FP64 on the device) ---- */

/* Static RPA dielectric matrix, RPA::calculate_epsilon_r
 * (xtp/src/libxtp/gwbse/rpa.cc:145-200): eps = 1 - 2 sum_{m occ} M_m^T diag(chi_m) M_m
 * with M_m = Mmn_[m].bottomRows(n_unocc) and the reference's chi at complex
 * frequency (freq_re, freq_im), eta = 1e-4.  rpa_energies: rpamax - rpamin + 1
 * values.  epsilon: auxsize x auxsize column-major (host). */
int bse_rpa_epsilon(const bse_mmn_desc *mmn, const double *const *mmn_slices,
                    const double *rpa_energies, int64_t rpatotal, int64_t homo,
                    int64_t rpamin, int64_t rpamax, double freq_re,
                    double freq_im, double *epsilon);

/* Ainv = A^-1 for a symmetric positive definite A (blocked Cholesky on the
 * device).  With A = eps this is the dense screening for
 * bse_op_create_dense_screening; it replaces the host eigen-decomposition in
 * BSE::SetupDirectInteractionOperator (xtp/src/libxtp/gwbse/bse.cc:188-204),
 * whose rotated-diagonal screening is mathematically the same operator. */
int bse_cholesky_inverse(int64_t n, const double *A, int64_t lda, double *Ainv,
                         int64_t ldi);

/* The screening of BSE::SetupDirectInteractionOperator (xtp/src/libxtp/gwbse/bse.cc:188-204)
 * as one dense matrix for any symmetric A (e.g. eps at a frequency beyond the first RPA
 * pole, where the Cholesky factorisation fails): A = U diag(lambda) U^T, W = U diag(w) U^T with
 * w = 1/lambda for lambda > cutoff (the reference uses 1e-8) and 0 otherwise.  The eigenproblem
 * is solved on the host, as in the reference; W is formed on the device. */
int bse_positive_inverse(int64_t n, const double *A, int64_t lda, double cutoff, double *W,
                         int64_t ldw);

/* TCMatrix_gwbse::MultiplyRightWithAuxMatrix (xtp/src/libxtp/threecenter.cc:54-65):
 * every slice M[m] <- M[m] * U (U auxsize x auxsize), in place on the host slices. */
int bse_mmn_multiply_right(const bse_mmn_desc *mmn, double *const *mmn_slices,
                           const double *U, int64_t ldu);

/* ---- Mmn producer (TCMatrix_gwbse::Fill, xtp/src/libxtp/threecenter.cc:79-95) ---- */

/* TCMatrix_gwbse::Fill3cMO (xtp/src/libxtp/libint2_calls.cc:595-651) with the AO
 * three-centre Coulomb integrals supplied by the caller in place of libint2:
 *   M(m, n, P) = sum_{mu,nu} C(mu, n) (P|mu nu) C(nu, m)
 * for m in [mmin, mmax], n in [nmin, nmax] of `mmn`; FP64 GEMMs on the device, batched over P.
 *   ao3c: auxsize column-major nbf x nbf symmetric matrices back to back,
 *         (P|mu nu) = ao3c[P * nbf * nbf + mu + nbf * nu].
 *   mo_coefficients: column-major nbf x nmo (dft_orbitals), leading dimension ldc.
 *   mmn_slices: msize output slices, each column-major nsize x auxsize (overwritten). */
int bse_mmn_fill_3c_mo(const bse_mmn_desc *mmn, double *const *mmn_slices, const double *ao3c, int64_t nbf,
                       const double *mo_coefficients, int64_t ldc, int64_t nmo);

/* AOCoulomb::Pseudo_InvSqrt (xtp/src/libxtp/aomatrices/aomatrix.cc:88-102): V^-1/2 over the
 * eigenvalues of V that are >= etol; `removed` (may be NULL) gets the number dropped. */
int bse_aux_pseudo_inv_sqrt(int64_t n, const double *V, int64_t ldv, double etol, double *out, int64_t ldo,
                            int64_t *removed);

/* AOCoulomb::Pseudo_InvSqrt_GWBSE (aomatrix.cc:53-86), the matrix TCMatrix_gwbse::Fill
 * multiplies Mmn with (threecenter.cc:86-93, etol 5e-7 there): S^-1/2 and
 * (S^-1/2 V S^-1/2)^-1/2 over the eigenvalues >= etol, result (V'^-1/2 S^-1/2)^T; `removed`
 * counts the functions dropped in both steps.  Eigenproblems on the host as in the reference,
 * products on the device. */
int bse_aux_pseudo_inv_sqrt_gwbse(int64_t n, const double *S, int64_t lds, const double *V, int64_t ldv,
                                  double etol, double *out, int64_t ldo, int64_t *removed);

/* Transition dipoles of BSE states from one spin block, Orbitals::CalcFreeTransition_Dipoles +
 * CalcCoupledTransition_Dipoles (xtp/src/libxtp/orbitals.cc:740-800 restricted singlets,
 * :804-877 combined UKS excitons), with the AO dipole matrices supplied by the caller in place
 * of libint2's AODipole (emultipole1 about the caller's origin):
 *   D_i = C[:, cmin : cmin + ctotal]^T dip_i C[:, vmin : vmin + vtotal]   (i = x, y, z)
 *   dipoles[3 s + i] (+)= prefactor sum_{v,c} (X + Y)(v ctotal + c, s) D_i(c, v)
 *   ao_dipoles: three column-major nbf x nbf matrices back to back (x, y, z);
 *   mo_coefficients: column-major nbf x nmo, leading dimension ldc;
 *   X, Y: the states' vectors (vtotal ctotal rows, leading dimension ldx, nstates columns);
 *         Y NULL for TDA states; a UKS block passes its rows of the combined vector;
 *   prefactor: -sqrt(2) for restricted singlets, -1 for each spin block of a UKS exciton;
 *   accumulate: 0 overwrites dipoles, 1 adds (the second spin block).
 * FP64 GEMMs on the device.  Oscillator strengths follow as f = 2/3 Omega |d|^2
 * (Orbitals::Oscillatorstrengths, orbitals.cc:645-673). */
int bse_transition_dipoles(const double *ao_dipoles, int64_t nbf, const double *mo_coefficients, int64_t ldc,
                           int64_t nmo, int64_t vmin, int64_t vtotal, int64_t cmin, int64_t ctotal,
                           const double *X, const double *Y, int64_t ldx, int64_t nstates, double prefactor,
                           int32_t accumulate, double *dipoles);

/* A dense FP64 symmetric matrix as an operator (the reference tests'
 * HermitianBlockOperator, test_davidson.cc:265-281).  b may be NULL; when
 * given, bse_ham_* use [[a, b], [-b, -a]]. */
int bse_dense_op_create(const double *a, const double *b, int64_t n,
                        int64_t lda, bse_handle **out);

int bse_op_destroy(bse_handle *h);

/* rows() == cols() of the (TDA) operator: vtotal * ctotal (or n). */
int bse_op_size(const bse_handle *h, int64_t *size);

/* Y = H(cqp,cx,cd,cd2) * X, host pointers, X and Y column-major dim x k.
 * Replaces BSE_OPERATOR::matmul (bse_operator.cc:39-119). */
int bse_op_matmul(bse_handle *h, int32_t cqp, int32_t cx, int32_t cd,
                  int32_t cd2, const double *X, int64_t ldx, int64_t k,
                  double *Y, int64_t ldy);

/* Same on device pointers, stream-ordered on `stream` (a cudaStream_t, NULL =
 * legacy default stream). */
int bse_op_matmul_device(bse_handle *h, int32_t cqp, int32_t cx, int32_t cd,
                         int32_t cd2, const double *dX, int64_t ldx, int64_t k,
                         double *dY, int64_t ldy, void *stream);

/* Allocation-free variant of bse_op_matmul_device.  It has no counterpart in
 * the reference.  It is for callers that cannot call cudaMalloc when they need
 * a product: code running while another component owns the device memory
 * through its own pool and forbids runtime allocations, or code that must not
 * take the device-wide synchronisation an allocation can cause inside a
 * pipelined solve.  The product is computed in FP64 (whatever precision the
 * handle was created with) with every temporary taken from one static 64 MiB
 * device array that each GPU loading this library holds until process exit;
 * no cudaMalloc, cudaFree or allocating library call is made.  Limits: a
 * request with Naux*k above 7 Mi doubles (Hx) or one column above 7 Mi doubles
 * of intermediate (Naux*v*c for Hd, Naux*v*v for Hd2) is rejected with
 * BSE_ERR_ARGUMENT.  The first call on a device looks up the array's device
 * address; make it before any stream capture.  All calls share the array:
 * calls that overlap on the GPU race, so serialise them on one stream. */
int bse_op_matmul_device_noalloc(bse_handle *h, int32_t cqp, int32_t cx,
                                 int32_t cd, int32_t cd2, const double *dX,
                                 int64_t ldx, int64_t k, double *dY,
                                 int64_t ldy, void *stream);

/* D = diagonal of H(cqp,cx,cd,cd2), host pointer of length size.
 * Replaces BSE_OPERATOR::diagonal (bse_operator.cc:133-175). */
int bse_op_diagonal(bse_handle *h, int32_t cqp, int32_t cx, int32_t cd,
                    int32_t cd2, double *D);
int bse_op_diagonal_device(bse_handle *h, int32_t cqp, int32_t cx, int32_t cd,
                           int32_t cd2, double *dD, void *stream);

/* HamiltonianOperator<A,B> product [[A, B], [-B, -A]] * X, X and Y column-major
 * (2*size) x k.  Replaces the product hook of bseoperator_btda.h:116-149. */
int bse_ham_matmul(bse_handle *h, const int32_t a_coef[4],
                   const int32_t b_coef[4], const double *X, int64_t ldx,
                   int64_t k, double *Y, int64_t ldy);

/* DavidsonSolver options (davidsonsolver.h:52-57, davidsonsolver.cc:101-170). */
typedef struct bse_davidson_options {
  int64_t iter_max;         /* set_iter_max (default 50) */
  double tolerance;         /* residual-norm tolerance (presets 1e-3/1e-4/1e-5/1e-9) */
  int64_t max_search_space; /* set_max_search_space (0 -> 5*neigen, as the reference) */
  int32_t correction;       /* 0 = DPR, 1 = OLSEN */
  int32_t update;           /* 0 = min, 1 = safe, 2 = max */
  int32_t matrix_type;      /* 0 = SYMM (Ritz), 1 = HAM (harmonic Ritz) */
  int32_t verbose;          /* print one line per iteration to stderr */
  /* Fields below have no counterpart in the reference; zero keeps its behaviour. */
  int32_t fp64_polish;      /* split-precision (BSE_PRECISION_MIXED) operators only: once the
                               split-precision iterations meet the tolerance (or their largest
                               residual has not halved in three iterations, or iter_max is
                               reached), the neigen Ritz vectors are re-applied with
                               FP64-accurate products and the iteration continues on that
                               basis until the residuals, formed from FP64-accurate products of
                               the Ritz vectors, meet the tolerance; the returned eigenvalues
                               are those Rayleigh quotients.  1: the FP64-accurate products are
                               the Ozaki slice products of BSE_PRECISION_SLICED; 2: FP64
                               DGEMM.  Ignored for FP64 and SLICED operators. */
  int32_t reserved;
  int64_t size_update;      /* trial vectors per iteration: 0 = getSizeUpdate of `update`
                               (davidsonsolver.cc:149-170); > 0 = that many (>= neigen) */
  int64_t initial_size;     /* without a guess: 0 = 2*neigen unit vectors (solve(A, neigen));
                               > 0 = that many (solve(A, neigen, size_initial_guess),
                               davidsonsolver.h:64-85) */
} bse_davidson_options;

typedef struct bse_davidson_result {
  int64_t iterations;      /* num_iterations() */
  int32_t info;            /* 0 = Success, 1 = NoConvergence (eigenpairs of unconverged roots zeroed) */
  int32_t polished;        /* 1 when the returned roots come from the FP64 polish */
  int64_t matvec_columns;  /* operator columns applied during the solve */
  double seconds_matvec;   /* device time in operator products */
  double seconds_total;    /* wall time of the solve */
  double max_residual;     /* largest residual norm of the neigen roots at return */
  int64_t fp64_columns;    /* columns applied with FP64 products by the polish */
  int64_t polish_iterations; /* iterations spent in the polish */
  double seconds_polish;   /* wall time of the polish */
} bse_davidson_result;

/*
 * DavidsonSolver::solve on the device (davidsonsolver.h:64-190): all vectors,
 * projections, Gram-Schmidt, residuals and corrections stay in HBM in FP64.
 *   SYMM: operator H(a_coef) (TDA singlet/triplet); b_coef ignored.
 *   HAM:  HamiltonianOperator [[A, B], [-B, -A]] with A = H(a_coef), B = H(b_coef).
 *   guess: NULL for the reference's unit-vector guess (2*neigen columns), else
 *          column-major (op size) x guess_cols (the solve(A, neigen, guess) overload).
 *   evals: neigen values; evecs: column-major (op size) x neigen, ldv >= op size
 *          (op size = size for SYMM, 2*size for HAM).  Either may be NULL.
 */
int bse_davidson_solve(bse_handle *h, const int32_t a_coef[4],
                       const int32_t b_coef[4],
                       const bse_davidson_options *opt, int64_t neigen,
                       const double *guess, int64_t guess_cols, double *evals,
                       double *evecs, int64_t ldv, bse_davidson_result *result);

/* ---- Diagnostics (no counterpart in the reference) ---- */

/* Stage indices of bse_op_profile_read. */
enum {
  BSE_STAGE_HQP = 0,
  BSE_STAGE_HX = 1,
  BSE_STAGE_HD_A = 2,
  BSE_STAGE_HD_B = 3,
  BSE_STAGE_HD2_A = 4,
  BSE_STAGE_HD2_B = 5,
  BSE_STAGE_TC_HD = 6,
  BSE_STAGE_TC_HX = 7,
  BSE_STAGE_TC_HD2 = 8,
  BSE_STAGE_TC_SPLIT = 9,
  BSE_STAGE_TC_HD_B = 10,
  BSE_STAGE_TC_HD2_B = 11,
  BSE_STAGE_COUNT = 12
};

/* enable != 0: record CUDA events around every stage of the product on its
 * launch stream and reset the counters; enable == 0: stop recording. */
int bse_op_profile(bse_handle *h, int32_t enable);
/* Accumulated device milliseconds and launches per stage since the last
 * bse_op_profile(h, 1); synchronises with the recorded events. */
int bse_op_profile_read(bse_handle *h, double *stage_ms, int64_t *stage_calls,
                        int32_t nstages);

/* Measured FP64 FMA throughput of the current device (TFLOP/s) from a short
 * register-resident FMA loop: the roofline denominator of the FP64 path. */
int bse_probe_fp64_tflops(double *tflops);

/* The device solver of the Davidson Ritz problems, exposed on its own: the lowest nw[i]
 * eigenpairs of each of njobs symmetric matrices, every matrix solved on the device in one
 * launch (one CTA each; FP64 Householder tridiagonalisation, FP32 bisection, FP64 inverse
 * iteration, back-transformation).  It takes the place of the Eigen::SelfAdjointEigenSolver
 * that DavidsonSolver::getRitz calls (xtp/src/libxtp/davidsonsolver.cc:221-239).  Host
 * pointers: T holds the matrices back to back (matrix i column-major m[i] x m[i], lower
 * triangle read); evals receives sum nw[i] values (ascending per matrix); evecs the m[i] x nw[i]
 * eigenvector blocks back to back (column-major, orthonormal columns, sign not fixed).
 * 1 <= nw[i] <= m[i] <= 3000.  phase_cycles (may be NULL): njobs x 4 SM clock cycles spent in
 * the tridiagonalisation, the bisection, the inverse iteration and the back-transformation. */
int bse_small_sym_eig(int64_t njobs, const int64_t *m, const int64_t *nw, const double *T,
                      double *evals, double *evecs, int64_t *phase_cycles);

/* The device solver of the harmonic-Ritz problem of the HAM Davidson, exposed on its own: the
 * real generalized problem T u = theta B u (m x m, general, column-major host arrays), the
 * reference's selection (the second member of each complex-conjugate pair dropped, an unpaired
 * complex eigenvalue an error; the nw largest real parts first) and its outputs: evecs (m x nw)
 * the real parts of the selected eigenvectors, each normalised, evals[c] = u_c^T T u_c.  It takes
 * the place of Eigen::GeneralizedEigenSolver and the selection in DavidsonSolver::getHarmonicRitz
 * (xtp/src/libxtp/davidsonsolver.cc:241-331).  Columns past the number of candidates are zero;
 * *selected (may be NULL) receives that number.  1 <= nw <= m <= 1024. */
int bse_small_gen_eig(int64_t m, int64_t nw, const double *T, const double *B, double *evals,
                      double *evecs, int64_t *selected);

/* The launch shapes the autotuner has chosen in this process (no counterpart in the reference):
 * a JSON array, one object per tuned kernel and tile width, with the chosen shape and every
 * candidate's measured time ([K box, operators per launch, streams, ms]).  The grouped dense products of
 * the lockstep batch are tuned on their first product round with at least 16 operators
 * (environment VGB_TC_AUTOTUNE=0 keeps the fixed shape).  buf (may be NULL) receives at most
 * cap - 1 characters and a terminating zero; *needed (may be NULL) the full length + 1. */
int bse_autotune_report(char *buf, int64_t cap, int64_t *needed);

/* ---- Adjoint (no counterpart in the reference; its forward twin is the
 * expectation-value analysis x^T H_part x of xtp/src/libxtp/gwbse/bse.cc:490-520) ----
 *
 * Hellmann-Feynman gradient of sum_k weights[k] * Omega_k for normalised
 * eigenvectors X (column-major dim x nroots, ldx) of the TDA operator
 * H(cqp, cx, cd, cd2) (for any coefficient set: the gradient of the quadratic forms):
 *   grad_mmn:       same layout as the Mmn slices given to bse_op_create
 *                   (msize x nsize x auxsize, slices back to back); entries
 *                   outside the BSE window are zero;
 *   grad_hqp:       (vt+ct) x (vt+ct) column-major gradient of the Hqp window;
 *   grad_screening: auxsize (diagonal epsilon_0_inv) or auxsize^2 (dense W).
 * Any output may be NULL.  Computed on the device: in FP64 for FP64 handles; handles with a
 * tensor-core engine (BSE_PRECISION_MIXED / _SLICED) form the two cc-block contractions
 * (2 Naux v c^2 flops per vector each) as FP64-accurate slice products (about 1e-10 of each
 * gradient block's norm from the FP64 gradient), the rest in FP64. */
int bse_op_eig_gradient(bse_handle *h, int32_t cqp, int32_t cx, int32_t cd,
                        int32_t cd2, const double *X, int64_t ldx,
                        int64_t nroots, const double *weights,
                        double *grad_mmn, double *grad_hqp,
                        double *grad_screening);

/* Full (non-TDA) BSE: gradient of sum_k weights[k] * Omega_k for eigenvectors (X_k, Y_k) of
 * [[A, B], [-B, -A]], A = H(a_coef), B = H(b_coef), normalised X^T X - Y^T Y = 1 (as
 * BSE::Solve_nonhermitian_Davidson returns them, bse.cc:315-360).  Omega is stationary in
 * z = (X, Y) for S z = Omega J z (S = [[A, B], [B, A]], J = diag(I, -I)), so
 * dOmega = X^T dA X + Y^T dA Y + 2 X^T dB Y for a symmetric dB, the sum
 * BSE::Analyze_eh_interaction forms for the full BSE (xtp/src/libxtp/gwbse/bse.cc:551-564); the
 * gradient with respect to single Mmn entries (which perturb B unsymmetrically) is that of
 * X^T (dB + dB^T) Y, the first-order change seen through the left eigenvector J z.
 * X, Y: host, dim x nroots (ldx); outputs as
 * bse_op_eig_gradient; grad_mmn also carries the entries M(c, v, P) that the Hd2 term of B reads.
 * Computed on the device, with the precision rule of bse_op_eig_gradient. */
int bse_op_eig_gradient_full(bse_handle *h, const int32_t a_coef[4], const int32_t b_coef[4],
                             const double *X, const double *Y, int64_t ldx, int64_t nroots,
                             const double *weights, double *grad_mmn, double *grad_hqp,
                             double *grad_screening);

/* The same gradients kept on the device in the operator's block layouts, so that a caller that
 * needs only some blocks (or feeds them to further device work) does not move the Mmn-shaped
 * gradient (8 * msize * nsize * auxsize bytes) to the host.  dX (and dY for the full BSE, NULL
 * for TDA, in which case b_coef is ignored): device, dim x nroots, leading dimension ldx;
 * weights: host.  Outputs (device, any may be NULL, overwritten):
 *   d_grad_vc  [P][v][c]  = dsum/dM(vmin + v, homo + 1 + c, P)       auxsize * dim
 *   d_grad_cv  [P][v][c]  = dsum/dM(homo + 1 + c, vmin + v, P)       auxsize * dim
 *   d_grad_vv  [P][v1][v] = dsum/dM(vmin + v1, vmin + v, P)          auxsize * vt * vt
 *   d_grad_cc  [P][c1][c] = dsum/dM(homo + 1 + c1, homo + 1 + c, P)  auxsize * ct * ct
 * (M(m, n, P) is row n - nmin of slice m - mmin, aux column P, as in bse_op_create).
 *   d_grad_hqp (vt + ct)^2 column-major window; d_grad_screening auxsize or auxsize^2.
 * Stream-ordered on `stream`; returns after the work completed. */
int bse_op_eig_gradient_device(bse_handle *h, const int32_t a_coef[4], const int32_t b_coef[4],
                               const double *dX, const double *dY, int64_t ldx, int64_t nroots,
                               const double *weights, double *d_grad_vc, double *d_grad_cv,
                               double *d_grad_vv, double *d_grad_cc, double *d_grad_hqp,
                               double *d_grad_screening, void *stream);

/* Many independent molecules (one handle each, e.g. of uneven BSE dimension),
 * bse_davidson_solve semantics (no guess, eigenvalues only).
 * nthreads <= 0: lockstep -- all molecules iterate together and every step of an
 *   iteration (tensor-core product stages, projections, Ritz vectors, DPR
 *   corrections, Gram-Schmidt) is one grouped launch over the molecules still
 *   iterating; needs BSE operator handles, matrix_type SYMM and DPR.
 * nthreads > 0: one independent solve per handle on that many host threads, each
 *   on its handle's stream with stream-ordered scratch (any handle and options).
 * evals: nhandles x neigen (row per molecule); infos / iterations: per molecule,
 * may be NULL.  No counterpart in the reference, which solves one molecule per
 * process (xtp_parallel farms jobs, xtp/src/libxtp/parallelxjobcalc.cc:52-74). */
int bse_davidson_solve_batch(bse_handle *const *handles, int64_t nhandles,
                             const int32_t a_coef[4], const int32_t b_coef[4],
                             const bse_davidson_options *opt, int64_t neigen,
                             double *evals, int32_t *infos,
                             int64_t *iterations, int32_t nthreads);

/* Thread-local text of the last error on this thread ("" if none). */
const char *bse_last_error(void);

/* Library version string. */
const char *bse_version(void);

#ifdef __cplusplus
}
#endif

#endif /* VOTCA_GB300_BSE_H */
