// Lockstep Davidson over many independent BSE operators (batch_davidson.cu).
#pragma once

#include <vector>

#include "bse_ops.cuh"

namespace vgb {

// Lowest neigen eigenvalues of every operator H_b(coef) (SYMM, DPR correction):
// evals[b * neigen + j]; infos[b] 0 = converged; iterations[b] as DavidsonSolver
// counts them.  All work is ordered on s.
void davidson_solve_batch(const std::vector<BseOperator *> &ops, const Coef &coef, int64_t neigen,
                          const bse_davidson_options &opt, double *evals, int32_t *infos,
                          int64_t *iterations, cudaStream_t s);

}  // namespace vgb
