"""Host-side mirror of VOTCA-XTP's DavidsonSolver; the solve runs on the GPU.

Option names and semantics follow xtp/include/votca/xtp/davidsonsolver.h:47-63
and xtp/src/libxtp/davidsonsolver.cc:101-170.  solve(op, neigen[, guess])
mirrors both solve overloads (davidsonsolver.h:64-190); the whole iteration
(projection, small eigenproblem, residuals, corrections, Gram-Schmidt,
restart) is done by bse_davidson_solve in libvotca_gb300.so.

solve_batch(ops, neigen) solves many independent molecules with the same
options concurrently (bse_davidson_solve_batch); the reference solves one
molecule per process.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .bse_operator import BSE_OPERATOR, DenseGpuOperator, HamiltonianOperator, _p

TOLERANCES = {"loose": 1e-3, "normal": 1e-4, "strict": 1e-5, "lapack": 1e-9}
CORRECTIONS = {"DPR": 0, "OLSEN": 1}
UPDATES = {"min": 0, "safe": 1, "max": 2}
MATRIX_TYPES = {"SYMM": 0, "HAM": 1}


class DavidsonSolver:
    def __init__(self, log=None):
        self.log_ = log
        self.iter_max_ = 50
        self.tol_ = 1e-4
        self.max_search_space_ = 0
        self.correction_ = 0
        self.update_ = 1
        self.matrix_type_ = 0
        self.verbose = False
        # no counterpart in the reference: FP64 polish of split-precision solves, trial vectors
        # per iteration (0 = getSizeUpdate), initial unit-vector guesses (0 = 2 * neigen)
        self.fp64_polish_ = 1
        self.block_size_ = 0
        self.initial_size_ = 0
        self.eigenvalues_ = None
        self.eigenvectors_ = None
        self.info_ = "NoConvergence"
        self.i_iter_ = 0
        self.result = None

    def set_iter_max(self, n):
        self.iter_max_ = int(n)

    def set_max_search_space(self, n):
        self.max_search_space_ = int(n)

    def set_tolerance(self, tol):
        if isinstance(tol, str):
            if tol not in TOLERANCES:
                raise RuntimeError(tol + " is not a valid Davidson tolerance")
            self.tol_ = TOLERANCES[tol]
        else:
            self.tol_ = float(tol)

    def set_correction(self, method):
        if method not in CORRECTIONS:
            raise RuntimeError(method + " is not a valid Davidson correction method")
        self.correction_ = CORRECTIONS[method]

    def set_size_update(self, s):
        if s not in UPDATES:
            raise RuntimeError(s + " is not a valid Davidson update")
        self.update_ = UPDATES[s]

    def set_fp64_polish(self, on):
        """Split-precision operators: re-evaluate the converged Ritz vectors with FP64-accurate
        products and iterate until those residuals meet the tolerance (on by default).  True or
        "sliced": Ozaki slice products on the tensor cores; "fp64": FP64 DGEMM; False: off."""
        if on == "fp64":
            self.fp64_polish_ = 2
        elif on == "sliced":
            self.fp64_polish_ = 1
        else:
            self.fp64_polish_ = 1 if on else 0

    def set_block_size(self, n):
        """Trial vectors added per iteration (>= neigen); 0 restores getSizeUpdate's rule."""
        self.block_size_ = int(n)

    def set_initial_size(self, n):
        """Unit-vector guesses of solve(A, neigen) (the size_initial_guess argument of the
        reference's overload, davidsonsolver.h:64-85); 0 means 2 * neigen."""
        self.initial_size_ = int(n)

    def set_matrix_type(self, mt):
        if mt not in MATRIX_TYPES:
            raise RuntimeError(mt + " is not a valid Davidson matrix type")
        self.matrix_type_ = MATRIX_TYPES[mt]

    def info(self):
        return self.info_

    def eigenvalues(self):
        return self.eigenvalues_

    def eigenvectors(self):
        return self.eigenvectors_

    def num_iterations(self):
        return self.i_iter_

    def _options(self):
        return _lib.bse_davidson_options(self.iter_max_, self.tol_, self.max_search_space_, self.correction_,
                                         self.update_, self.matrix_type_, int(self.verbose),
                                         int(self.fp64_polish_), 0, self.block_size_, self.initial_size_)

    def solve_batch(self, ops, neigen, nthreads=0):
        """Lowest neigen eigenvalues of every operator in ops (BSE_OPERATORs with one
        coefficient set, or DenseGpuOperators).  nthreads=0: all molecules iterate in
        lockstep, every step one grouped launch (BSE operators, DPR); nthreads>0: one
        independent solve per molecule on that many host threads (any operator/option).
        Returns (evals [len(ops) x neigen], info per molecule, iterations per molecule)."""
        ops = list(ops)
        n = len(ops)
        if n == 0:
            return np.zeros((0, neigen)), [], np.zeros(0, dtype=np.int64)
        if self.matrix_type_ != MATRIX_TYPES["SYMM"]:
            raise RuntimeError("DavidsonSolver.solve_batch: only SYMM operators are batched")
        first = ops[0]
        if isinstance(first, BSE_OPERATOR):
            coef = first.coef
            if any(not isinstance(o, BSE_OPERATOR) or o.coef != coef for o in ops):
                raise TypeError("solve_batch: all operators must share one BSE_OPERATOR coefficient set")
            L = first.ctx._L
            handles = [o.ctx.handle for o in ops]
        elif isinstance(first, DenseGpuOperator):
            if any(not isinstance(o, DenseGpuOperator) for o in ops):
                raise TypeError("solve_batch: mixed operator kinds")
            coef = (0, 0, 0, 0)
            L = first._L
            handles = [o.handle for o in ops]
        else:
            raise TypeError("DavidsonSolver.solve_batch needs GPU operators")
        harr = (ctypes.c_void_p * n)(*[h.value if isinstance(h, ctypes.c_void_p) else h for h in handles])
        a = (ctypes.c_int32 * 4)(*coef)
        b = (ctypes.c_int32 * 4)(0, 0, 0, 0)
        opt = self._options()
        evals = np.zeros((n, neigen))
        infos = (ctypes.c_int32 * n)()
        iters = (ctypes.c_int64 * n)()
        _lib.check(L.bse_davidson_solve_batch(harr, n, a, b, ctypes.byref(opt), neigen, _p(evals), infos, iters,
                                              int(nthreads)))
        info = ["Success" if infos[i] == 0 else "NoConvergence" for i in range(n)]
        return evals, info, np.array(iters[:], dtype=np.int64)

    def solve(self, A, neigen, initial_guess=None):
        if isinstance(A, HamiltonianOperator):
            if isinstance(A.A_, DenseGpuOperator):
                L, h = A.A_._L, A.A_.handle
                a = b = (ctypes.c_int32 * 4)(0, 0, 0, 0)
            else:
                L, h = A.A_.ctx._L, A.A_.ctx.handle
                a = (ctypes.c_int32 * 4)(*A.A_.coef)
                b = (ctypes.c_int32 * 4)(*A.B_.coef)
            n = A.rows()
        elif isinstance(A, (BSE_OPERATOR,)):
            L, h = A.ctx._L, A.ctx.handle
            a = (ctypes.c_int32 * 4)(*A.coef)
            b = (ctypes.c_int32 * 4)(0, 0, 0, 0)
            n = A.rows()
        elif isinstance(A, DenseGpuOperator):
            L, h = A._L, A.handle
            a = b = (ctypes.c_int32 * 4)(0, 0, 0, 0)
            n = A.rows()
        else:
            raise TypeError("DavidsonSolver.solve needs a GPU operator")
        opt = self._options()
        evals = np.zeros(neigen)
        evecs = np.zeros((n, neigen), order="F")
        res = _lib.bse_davidson_result()
        if initial_guess is not None:
            g = np.asfortranarray(initial_guess, dtype=np.float64)
            if g.shape[0] != n:
                raise RuntimeError("DavidsonSolver::solve initial_guess has wrong number of rows.")
            gp, gc = _p(g), g.shape[1]
        else:
            gp, gc = None, 0
        _lib.check(L.bse_davidson_solve(h, a, b, ctypes.byref(opt), neigen, gp, gc, _p(evals), _p(evecs), n,
                                        ctypes.byref(res)))
        self.eigenvalues_ = evals
        self.eigenvectors_ = evecs
        self.info_ = "Success" if res.info == 0 else "NoConvergence"
        self.i_iter_ = res.iterations
        self.result = res
        return evals, evecs
