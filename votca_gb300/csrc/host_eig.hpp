// Small dense eigensolvers for the Davidson projected problems (host, FP64).
#pragma once

#include <cstdint>
#include <vector>

namespace vgb {

// Symmetric eigen-decomposition of the n x n column-major matrix A:
// eigenvalues ascending, eigenvectors as columns of V (n x n, column-major).
// Householder tridiagonalisation followed by the implicit-shift QL iteration.
// Returns false if the QL iteration does not converge.
bool sym_eig(int64_t n, const double *A, std::vector<double> &evals, std::vector<double> &V);

// Real generalized eigenproblem T x = lambda B x (both n x n, column-major,
// general).  Returns real and imaginary parts of the eigenvalues and the real
// eigenvectors as columns (for a complex pair (i, i+1) column i holds the real
// part and column i+1 the imaginary part, LAPACK-style).  Reduces to the
// standard problem B^-1 T (LU with partial pivoting), then Hessenberg
// reduction and the Francis double-shift QR iteration.  Returns false on
// failure (singular B or no convergence).
bool gen_eig(int64_t n, const double *T, const double *B, std::vector<double> &wr,
             std::vector<double> &wi, std::vector<double> &V);

}  // namespace vgb
