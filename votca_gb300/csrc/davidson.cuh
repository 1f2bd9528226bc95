// Block Davidson eigensolver with every vector operation in HBM (FP64).
#pragma once

#include "bse_ops.cuh"

namespace vgb {

struct DavidsonOutput {
  std::vector<double> evals;  // neigen
  int64_t iterations = 0;
  int info = 1;  // 0 success, 1 no convergence
  int64_t matvec_columns = 0;
  double seconds_matvec = 0.0, seconds_total = 0.0;
  std::vector<double> history_resnorm;  // max residual of the first neigen roots, per iteration
  double max_residual = 0.0;            // of the neigen roots at return
  int polished = 0;                     // roots from the FP64 polish
  int64_t fp64_columns = 0, polish_iterations = 0;
  double seconds_polish = 0.0;
};

// Mirrors DavidsonSolver::solve (xtp/include/votca/xtp/davidsonsolver.h:64-190,
// xtp/src/libxtp/davidsonsolver.cc).  evecs_dev (n x neigen, ld n) receives the
// normalised eigenvectors on the device; may be nullptr.
void davidson_solve(DeviceOperator &A, int64_t neigen, const bse_davidson_options &opt,
                    const double *host_guess, int64_t guess_cols, double *evecs_dev,
                    DavidsonOutput &out, cudaStream_t s);

}  // namespace vgb
