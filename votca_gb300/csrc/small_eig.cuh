// Small dense symmetric eigenproblems on the device (FP64), one CTA per problem.
//
// The Davidson projected matrices T = V^T A V (m up to a few hundred) are solved where they are
// formed, so the search space never leaves HBM: the Ritz problem of getRitz
// (xtp/src/libxtp/davidsonsolver.cc:221-239, Eigen::SelfAdjointEigenSolver there) for the
// single solve and for every molecule of a lockstep batch in one launch.
//
// Method (all published textbook steps, no library code):
//   1. Householder reduction to tridiagonal form, lower triangle, in shared memory when the
//      matrix fits (else in the job's global scratch): per column one reflector
//      H = I - tau v v^T (v_0 = 1), p = tau A v, w = p - (tau/2)(p.v) v, A -= v w^T + w v^T.
//   2. The wanted (lowest nw) eigenvalues of the tridiagonal matrix by bisection on the Sturm
//      count in FP32, one thread per eigenvalue (FP32 runs at 64x the FP64 rate of GB300).
//   3. Eigenvectors by inverse iteration in FP64 with the tridiagonal LU with partial
//      pivoting: two steps at the FP32 shift, then the FP64 Rayleigh quotient as the shift
//      and two more steps (Rayleigh quotient iteration).  Eigenvalues closer than 1e-5 of the
//      spectral radius form a cluster: its vectors are computed one after another, each step
//      orthogonalised against the earlier members (modified Gram-Schmidt), then a
//      Rayleigh-Ritz step on the cluster (cyclic Jacobi on Z_c^T T Z_c) separates them.
//   4. Back-transformation U = Q Z with the stored reflectors, one warp per eigenvector.
// Eigenvalues are returned ascending (as SelfAdjointEigenSolver orders them), eigenvectors
// orthonormal; the sign of each eigenvector is not fixed (neither is Eigen's).
#pragma once

#include "common.cuh"

namespace vgb {

struct SymEigJob {
  const double *T = nullptr;  // m x m symmetric, column-major; the lower triangle is read
  int64_t ldt = 0;
  int64_t m = 0;
  int64_t nw = 0;             // lowest nw eigenpairs, 1 <= nw <= m
  double *U = nullptr;        // m x nw eigenvectors (output), leading dimension ldu >= m
  int64_t ldu = 0;
  double *lam = nullptr;      // nw eigenvalues ascending (output)
  double *work = nullptr;     // sym_eig_work_doubles(m, nw) doubles of device scratch
  int *info = nullptr;        // may be null; set nonzero when the job's sizes are invalid
  long long *clocks = nullptr;  // may be null; 5 SM clock readings at the phase boundaries
};

// Device scratch one job needs.
int64_t sym_eig_work_doubles(int64_t m, int64_t nw);
// Largest m a job may have (the vector part of the shared-memory layout must fit).
constexpr int64_t kSymEigMaxM = 3000;

// Solve every job (one CTA each), stream-ordered on s.
void sym_eig_device(const SymEigJob *jobs, int64_t njobs, cudaStream_t s);

// The harmonic-Ritz problem of the HAM Davidson (gen_eig.cu): T u = theta B u for general m x m
// T, B; the reference's selection (complex partners dropped, the nw largest real parts) and
// its outputs: U = the real parts of those eigenvectors, normalised, lam = diag(U^T T U).
struct GenEigJob {
  const double *T = nullptr, *B = nullptr;  // column-major, leading dimension ldt
  int64_t ldt = 0;
  int64_t m = 0;
  int64_t nw = 0;        // 1 <= nw <= m
  double *U = nullptr;   // m x nw (leading dimension ldu >= m), output
  int64_t ldu = 0;
  double *lam = nullptr; // nw, output (zero past the number of candidates)
  double *work = nullptr;  // gen_eig_work_doubles(m, nw) doubles
  int *info = nullptr;   // two ints: [0] 0 ok, 1 invalid sizes, 2 B singular or B^-1 T not finite,
                         // 3 QR iteration without convergence, 4 a complex eigenvalue without
                         // partner (its index in [1]); on success [1] = pairs selected
};
constexpr int64_t kGenEigMaxM = 1024;
int64_t gen_eig_work_doubles(int64_t m, int64_t nw);
void gen_eig_device(const GenEigJob *jobs, int64_t njobs, cudaStream_t s);
// O (m x r, ldo) = an orthonormal basis of the columns of U (modified Gram-Schmidt twice, one CTA);
// the restart of the HAM Davidson (DavidsonSolver::qr, davidsonsolver.cc:480-488).
void orthonormalise_device(const double *U, int64_t ldu, int64_t m, int64_t r, double *O, int64_t ldo,
                           cudaStream_t s);
// The FP64 polish of a HAM solve reduces its projected pencil (S, J) (S symmetric positive
// definite, lower triangle read; J symmetric, full; ld) on the device: W (3 m^2 doubles) receives
// L = chol(S), L^-1 J and Mneg = -L^-1 J L^-T (its leading m^2 x 3 block, each ld m); *status = 1
// when S is not positive definite.  After sym_eig_device on Mneg (np lowest: the largest mu),
// pencil_finish_device returns lam = 1 / mu and U = L^-T z (m x np, ld m); *status = 2 when fewer
// than np of the mu are positive.
void pencil_reduce_device(const double *S, const double *J, int64_t ld, int64_t m, double *W, int *status,
                          cudaStream_t s);
void pencil_finish_device(const double *W, int64_t m, const double *nu, const double *Z, int64_t np, double *U,
                          double *lam, int *status, cudaStream_t s);

}  // namespace vgb
