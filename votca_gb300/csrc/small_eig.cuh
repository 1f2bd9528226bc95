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

}  // namespace vgb
