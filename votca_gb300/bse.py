"""Mirror of the BSE solve drivers of VOTCA-XTP (xtp/src/libxtp/gwbse/bse.cc).

  solve_hermitian             BSE::solve_hermitian, bse.cc:266-293
  solve_nonhermitian_davidson BSE::Solve_nonhermitian_Davidson, bse.cc:315-360
  full_bse_ranked_guess       BuildFullBSEXRankedInitialGuess,
                              xtp/include/votca/xtp/bse_initialization.h:47-92

The Davidson iteration itself runs on the GPU (bse_davidson_solve).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .bse_operator import HamiltonianOperator
from .davidson import DavidsonSolver


@dataclass
class DavidsonOptions:
    """The BSE Davidson knobs of xtp/share/xtp/xml/subpackages/gwbse.xml."""
    davidson_correction: str = "DPR"
    davidson_tolerance: object = "normal"  # preset name or a number
    davidson_update: str = "safe"
    davidson_maxiter: int = 50
    nmax: int = 5


def _solver(opt: DavidsonOptions):
    ds = DavidsonSolver()
    ds.set_correction(opt.davidson_correction)
    ds.set_tolerance(opt.davidson_tolerance)
    ds.set_size_update(opt.davidson_update)
    ds.set_iter_max(opt.davidson_maxiter)
    ds.set_max_search_space(10 * opt.nmax)
    return ds


def solve_hermitian(h, opt: DavidsonOptions):
    ds = _solver(opt)
    evals, evecs = ds.solve(h, opt.nmax)
    return evals, evecs, ds


def full_bse_ranked_guess(adiag, bdiag, nroots):
    adiag = np.asarray(adiag, dtype=np.float64)
    bdiag = np.asarray(bdiag, dtype=np.float64)
    if adiag.size != bdiag.size:
        raise RuntimeError("BuildFullBSEXRankedInitialGuess: size mismatch.")
    n = adiag.size
    nguess = min(n, max(4 * nroots, 8))
    omega = np.sqrt(np.maximum(0.0, (adiag - bdiag) * (adiag + bdiag)))
    order = sorted(range(n), key=lambda i: (omega[i], adiag[i]))
    guess = np.zeros((2 * n, nguess), order="F")
    for col in range(nguess):
        guess[order[col], col] = 1.0
    return guess


def solve_nonhermitian_davidson(A, B, opt: DavidsonOptions):
    """Returns (eigenvalues, X, Y, solver) with |X|^2 - |Y|^2 = 1 per root."""
    hop = HamiltonianOperator(A, B)
    ds = _solver(opt)
    ds.set_matrix_type("HAM")
    guess = full_bse_ranked_guess(A.diagonal(), B.diagonal(), opt.nmax)
    evals, evecs = ds.solve(hop, opt.nmax, guess)
    n = A.rows()
    X, Y = evecs[:n], evecs[n:]
    with np.errstate(invalid="ignore", divide="ignore"):
        s = np.sqrt(1.0 / (np.sum(X * X, axis=0) - np.sum(Y * Y, axis=0)))
    return evals, X * s, Y * s, ds
