"""NumPy restatement of VOTCA-XTP's DavidsonSolver (TEST INFRASTRUCTURE ONLY).

The shipped library never imports this module.  Tests, the smoke check and the
CPU-baseline leg of the benchmark use it as the reference for comparisons.

Follows, step by step:
  DavidsonSolver::solve (both overloads)     xtp/include/votca/xtp/davidsonsolver.h:64-190
  updateProjection                            davidsonsolver.h:239-280
  set_tolerance / getSizeUpdate               xtp/src/libxtp/davidsonsolver.cc:122-170
  argsort / setupInitialEigenvectors          davidsonsolver.cc:172-206
  getRitz (SelfAdjointEigenSolver, ascending) davidsonsolver.cc:221-239
  getHarmonicRitz (GeneralizedEigenSolver)    davidsonsolver.cc:241-332
  checkConvergence / extendProjection         davidsonsolver.cc:347-378
  computeCorrectionVector / dpr / olsen       davidsonsolver.cc:389-436
  gramschmidt (two passes, throws on lin.dep) davidsonsolver.cc:442-478
  qr (Householder Q, thin)                    davidsonsolver.cc:480-488
  restart                                     davidsonsolver.cc:490-513
  storeConvergedData / storeNotConvergedData  davidsonsolver.cc:515-555
  HamiltonianOperator diagonal [D_A; -D_A]    xtp/include/votca/xtp/bseoperator_btda.h:81-87
  BuildFullBSEXRankedInitialGuess             xtp/include/votca/xtp/bse_initialization.h:47-92
  BSE::Solve_nonhermitian_Davidson X/Y norm   xtp/src/libxtp/gwbse/bse.cc:315-360

numpy.linalg.eigh stands in for Eigen::SelfAdjointEigenSolver (both return
ascending eigenvalues); scipy.linalg.eig(T, B) stands in for
Eigen::GeneralizedEigenSolver (eigenvector scaling differs, but the reference
re-normalises the real parts before use).
"""
from __future__ import annotations

import numpy as np

TOLERANCES = {"loose": 1e-3, "normal": 1e-4, "strict": 1e-5, "lapack": 1e-9}


class DavidsonNotConverged(Exception):
    pass


class DavidsonOracle:
    def __init__(self):
        self.iter_max = 50
        self.tol = 1e-4
        self.max_search_space = 0
        self.correction = "DPR"
        self.update = "SAFE"
        self.matrix_type = "SYMM"
        self.info = "NoConvergence"
        self.i_iter = 0
        self.eigenvalues = None
        self.eigenvectors = None
        self.restart_size = 0
        self.Adiag = None
        self.matvec_columns = 0  # number of operator columns applied (bookkeeping)

    # -- options (davidsonsolver.cc:101-147) --
    def set_tolerance(self, tol):
        if isinstance(tol, str):
            if tol not in TOLERANCES:
                raise RuntimeError(tol + " is not a valid Davidson tolerance")
            self.tol = TOLERANCES[tol]
        else:
            self.tol = float(tol)

    def set_correction(self, method):
        if method not in ("DPR", "OLSEN"):
            raise RuntimeError(method + " is not a valid Davidson correction method")
        self.correction = method

    def set_size_update(self, s):
        m = {"min": "MIN", "safe": "SAFE", "max": "MAX"}
        if s not in m:
            raise RuntimeError(s + " is not a valid Davidson update")
        self.update = m[s]

    def set_matrix_type(self, mt):
        if mt not in ("HAM", "SYMM"):
            raise RuntimeError(mt + " is not a valid Davidson matrix type")
        self.matrix_type = mt

    def size_update(self, neigen):
        if self.update == "MIN":
            return neigen
        if self.update == "SAFE":
            return int(1.5 * neigen) if neigen < 20 else neigen + 10
        return 2 * neigen

    # -- pieces --
    @staticmethod
    def argsort(v):
        return np.argsort(v, kind="stable")

    def setup_initial_eigenvectors(self, size_initial_guess):
        n = self.Adiag.size
        guess = np.zeros((n, size_initial_guess))
        idx = self.argsort(self.Adiag)
        if self.matrix_type == "SYMM":
            for j in range(size_initial_guess):
                guess[idx[j], j] = 1.0
        else:
            ind0 = n // 2
            for j in range(size_initial_guess):
                guess[idx[ind0 + j], j] = 1.0
        return guess

    @staticmethod
    def _normalize_cols(Q):
        """Eigen's normalize(): a zero column is left unchanged."""
        n = np.linalg.norm(Q, axis=0)
        Q /= np.where(n > 0, n, 1.0)

    def gramschmidt(self, Q, nstart):
        norms = np.linalg.norm(Q[:, nstart:], axis=0)
        for rep in range(2):
            if nstart > 0:
                L = Q[:, :nstart]
                Q[:, nstart:] -= L @ (L.T @ Q[:, nstart:])
                self._normalize_cols(Q[:, nstart:])
            for j in range(nstart + 1, Q.shape[1]):
                rng = j - nstart
                M = Q[:, nstart:j]
                Q[:, j] -= M @ (M.T @ Q[:, j])
                if rep == 1 and np.linalg.norm(Q[:, j]) <= 1e-12 * norms[rng]:
                    raise RuntimeError("Linear dependencies in Gram-Schmidt.")
                self._normalize_cols(Q[:, j:j + 1])
        return Q

    def dpr(self, r, lam):
        with np.errstate(divide="ignore", invalid="ignore"):
            return -r / (self.Adiag - lam)

    def correction_vector(self, q, lam, r):
        if self.correction == "DPR":
            c = self.dpr(r, lam)
        else:
            delta = self.dpr(r, lam)
            num = -q @ delta
            denom = -q @ self.dpr(q, lam)
            c = delta + (num / denom) * q
        c = np.where(np.isfinite(c), c, 0.0)
        return c

    @staticmethod
    def qr(A):
        q, _ = np.linalg.qr(A, mode="reduced")
        # Householder Q times the thin identity; column signs follow the
        # Householder convention of the reference (R with non-positive
        # leading diagonal is not normalised): any sign choice spans the same
        # space, which is all restart uses.
        return q

    def get_ritz(self, proj):
        evals, evecs = np.linalg.eigh(proj["T"])
        needed = min(proj["T"].shape[1], max(self.restart_size, proj["size_update"]))
        lam = evals[:needed]
        U = evecs[:, :needed]
        q = proj["V"] @ U
        res = proj["AV"] @ U - q * lam
        return dict(lam=lam, U=U, q=q, res=res)

    def get_harmonic_ritz(self, proj):
        import scipy.linalg

        w, vr = scipy.linalg.eig(proj["T"], proj["B"])
        n = w.size
        pairs = []
        for i in range(n):
            if w[i].imag != 0:
                found = False
                for p in pairs:
                    if p[1] > -1:
                        continue
                    if abs(w[p[0]].real - w[i].real) < 1e-9 and abs(w[p[0]].imag + w[i].imag) < 1e-9:
                        p[1] = i
                        found = True
                if not found:
                    pairs.append([i, -1])
        for p in pairs:
            if p[1] < 0:
                raise RuntimeError(f"Eigenvalue:{p[0]} is complex but has no partner.")
        second = {p[1] for p in pairs}
        evals, evecs = [], []
        for i in range(n):
            if i in second:
                continue
            evals.append(w[i].real)
            v = vr[:, i].real.copy()
            v /= np.linalg.norm(v)
            evals_v = v
            evecs.append(evals_v)
        evals = np.array(evals)
        evecs = np.array(evecs).T
        needed = min(proj["T"].shape[1], max(self.restart_size, proj["size_update"]))
        idx = self.argsort(evals)[::-1][:needed]
        U = evecs[:, idx]
        lam = np.diag(U.T @ proj["T"] @ U).copy()
        q = proj["V"] @ U
        res = proj["AV"] @ U - q * lam
        return dict(lam=lam, U=U, q=q, res=res)

    def update_projection(self, A, proj):
        if self.i_iter == 0:
            proj["AV"] = A(proj["V"])
            self.matvec_columns += proj["V"].shape[1]
            proj["T"] = proj["V"].T @ proj["AV"]
            if self.matrix_type == "HAM":
                proj["AAV"] = A(proj["AV"])
                self.matvec_columns += proj["V"].shape[1]
                proj["B"] = proj["V"].T @ proj["AAV"]
        else:
            old = proj["AV"].shape[1]
            new = proj["V"].shape[1]
            nvec = new - old
            Vn = proj["V"][:, old:]
            AVn = A(Vn)
            self.matvec_columns += nvec
            proj["AV"] = np.concatenate([proj["AV"], AVn], axis=1)
            T = np.zeros((new, new))
            T[:old, :old] = proj["T"]
            T[:, old:] = proj["V"].T @ AVn
            if self.matrix_type == "SYMM":
                T[old:, :old] = T[:old, old:].T
            else:
                T[old:, :old] = Vn.T @ proj["AV"][:, :old]
                AAVn = A(AVn)
                self.matvec_columns += nvec
                proj["AAV"] = np.concatenate([proj["AAV"], AAVn], axis=1)
                B = np.zeros((new, new))
                B[:old, :old] = proj["B"]
                B[:, old:] = proj["V"].T @ AAVn
                B[old:, :old] = Vn.T @ proj["AAV"][:, :old]
                proj["B"] = B
            proj["T"] = T

    def extend_projection(self, rep, proj):
        conv = proj["root_converged"]
        nupdate = int(np.count_nonzero(~conv))
        old = proj["V"].shape[1]
        newcols = []
        for j in range(proj["size_update"]):
            if conv[j]:
                continue
            wv = self.correction_vector(rep["q"][:, j], rep["lam"][j], rep["res"][:, j])
            newcols.append(wv / np.linalg.norm(wv))
        V = np.concatenate([proj["V"], np.array(newcols).T], axis=1) if newcols else proj["V"]
        self.gramschmidt(V, V.shape[1] - nupdate)
        proj["V"] = V
        del old
        return nupdate

    def restart(self, rep, proj, newvectors):
        rs = self.restart_size
        V = proj["V"]
        newV = np.empty((V.shape[0], newvectors + rs))
        newV[:, rs:] = V[:, V.shape[1] - newvectors:]
        if self.matrix_type == "SYMM":
            newV[:, :rs] = rep["q"][:, :rs]
            proj["AV"] = proj["AV"] @ rep["U"][:, :rs]
        else:
            ortho = self.qr(rep["U"][:, :rs])
            newV[:, :rs] = V[:, : V.shape[1] - newvectors] @ ortho
            proj["AV"] = proj["AV"] @ ortho
            proj["AAV"] = proj["AAV"] @ ortho
            proj["B"] = newV[:, :rs].T @ proj["AAV"]
        proj["T"] = newV[:, :rs].T @ proj["AV"]
        proj["V"] = newV

    def store(self, rep, neigen):
        self.eigenvalues = rep["lam"][:neigen].copy()
        ev = rep["q"][:, :neigen].copy()
        self.eigenvectors = ev / np.linalg.norm(ev, axis=0)

    # -- driver --
    def solve(self, A, Adiag, neigen, size_initial_guess=0, initial_guess=None):
        """A: callable X (n x k) -> A @ X.  Adiag: operator diagonal."""
        if self.max_search_space < neigen:
            self.max_search_space = neigen * 5
        n = Adiag.size
        if self.max_search_space > n:
            self.max_search_space = n
        self.Adiag = np.asarray(Adiag, dtype=np.float64)
        proj = {}
        if initial_guess is None:
            if size_initial_guess == 0:
                size_initial_guess = 2 * neigen
            self.restart_size = size_initial_guess
            proj["V"] = self.setup_initial_eigenvectors(size_initial_guess)
        else:
            if initial_guess.shape[0] != n:
                raise RuntimeError("DavidsonSolver::solve initial_guess has wrong number of rows.")
            if initial_guess.shape[1] < neigen:
                raise RuntimeError("DavidsonSolver::solve initial_guess has fewer columns than neigen.")
            self.restart_size = min(initial_guess.shape[1], self.max_search_space)
            V = np.array(initial_guess, dtype=np.float64, copy=True)
            self.gramschmidt(V, 0)
            proj["V"] = V
        proj["size_update"] = self.size_update(neigen)
        proj["root_converged"] = np.zeros(proj["size_update"], dtype=bool)
        self.history = []
        for self.i_iter in range(self.iter_max):
            self.update_projection(A, proj)
            rep = self.get_harmonic_ritz(proj) if self.matrix_type == "HAM" else self.get_ritz(proj)
            rn = np.linalg.norm(rep["res"], axis=0)
            conv = rn[: proj["size_update"]] < self.tol
            if conv.size < proj["size_update"]:
                conv = np.concatenate([conv, np.zeros(proj["size_update"] - conv.size, bool)])
            proj["root_converged"] = conv
            converged = bool(conv[:neigen].all())
            self.history.append((proj["V"].shape[1], float(rn[:neigen].max())))
            last = self.i_iter == self.iter_max - 1
            if converged:
                self.store(rep, neigen)
                self.info = "Success"
                break
            if last:
                self.store(rep, neigen)
                for i in range(neigen):
                    if not conv[i]:
                        self.eigenvalues[i] = 0.0
                        self.eigenvectors[:, i] = 0.0
                self.info = "NoConvergence"
                break
            ext = self.extend_projection(rep, proj)
            if proj["V"].shape[1] > self.max_search_space:
                self.restart(rep, proj, ext)
        return self.eigenvalues, self.eigenvectors


def init_matrix(n, eps):
    """test_davidson.cc:42-56: diagonal sqrt(i+1), off-diagonal eps/(j-i)^2."""
    i = np.arange(n)
    d = np.abs(i[:, None] - i[None, :]).astype(np.float64)
    with np.errstate(divide="ignore"):
        A = eps / d**2
    A[i, i] = np.sqrt(1.0 + i)
    return A


def ham_diagonal(adiag):
    """HamiltonianOperator::get_diagonal, bseoperator_btda.h:81-87."""
    return np.concatenate([adiag, -adiag])


def full_bse_ranked_guess(adiag, bdiag, nroots):
    """BuildFullBSEXRankedInitialGuess, bse_initialization.h:47-92."""
    if adiag.size != bdiag.size:
        raise RuntimeError("BuildFullBSEXRankedInitialGuess: size mismatch.")
    n = adiag.size
    nguess = min(n, max(4 * nroots, 8))
    omega = np.sqrt(np.maximum(0.0, (adiag - bdiag) * (adiag + bdiag)))
    order = np.lexsort((adiag, omega))  # primary omega, secondary a
    guess = np.zeros((2 * n, nguess))
    for col in range(nguess):
        guess[order[col], col] = 1.0
    return guess


def normalize_xy(evecs, dim):
    """bse.cc:340-350: scale so that |X|^2 - |Y|^2 = 1."""
    X = evecs[:dim]
    Y = evecs[dim:]
    s = np.sqrt(1.0 / (np.sum(X * X, axis=0) - np.sum(Y * Y, axis=0)))
    return X * s, Y * s
