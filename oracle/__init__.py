"""CPU oracle for the BSE hot path (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py may
import this package, and only to compare results against or as the timed CPU
reference.  The product package (votca_gb300) never imports it.

  bse_oracle.c        restated BSE_OPERATOR loop nest + diagonal + factorised form
                      + HamiltonianOperator product (ctypes-loaded below)
  davidson_oracle.py  restated DavidsonSolver (SYMM Ritz and HAM harmonic Ritz)
  rpa_oracle.py       restated RPA epsilon and the eigen-rotation screening
  uks_oracle.py       restated BSE_OPERATOR_UKS blocks
  threecenter_oracle.py   restated Fill3cMO and the auxiliary metrics
  gaussian_integrals.py   McMurchie-Davidson AO integrals for the golden methane case
  orbitals_oracle.py  restated transition dipoles and oscillator strengths
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libbse_oracle.so")
_lib = None

# BSE_OPERATOR<cqp, cx, cd, cd2> coefficient sets, bse_operator.h:79-87
OPERATORS = {
    "singlet": (1, 2, 1, 0),      # SingletOperator_TDA
    "triplet": (1, 0, 1, 0),      # TripletOperator_TDA
    "singlet_b": (0, 2, 0, 1),    # SingletOperator_BTDA_B
    "hqp": (1, 0, 0, 0),          # HqpOperator
    "hx": (0, 1, 0, 0),           # HxOperator
    "hd": (0, 0, 1, 0),           # HdOperator
    "hd2": (0, 0, 0, 1),          # Hd2Operator
}


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
            os.path.join(_HERE, "bse_oracle.c")
        ):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.POINTER(ctypes.c_double)
        I = ctypes.c_longlong
        common = [P, I, I, I, P, P, I, I, I, I, I, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.oracle_bse_matmul_ref.argtypes = common + [P, I, I, P, I, I, I, I, I]
        L.oracle_bse_matmul_fact.argtypes = common + [P, I, I, P, I]
        L.oracle_bse_matmul_rows.argtypes = common + [P, I, I, ctypes.POINTER(ctypes.c_longlong), I, P]
        L.oracle_bse_diagonal.argtypes = common + [P]
        L.oracle_ham_matmul.argtypes = [P, I, I, I, P, P, I, I, I, I, I,
                                        ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                        P, I, P, ctypes.c_int]
        L.oracle_num_threads.restype = ctypes.c_int
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class BSEProblem:
    """Inputs of one BSE_OPERATOR in the reference's conventions.

    mmn:  (nm, naux, nn) C-order array == the reference's vector of nm column-major
          [nn x naux] slices stored back to back: M(m, n, P) = mmn[m, P, n].
    w:    epsilon_0_inv (naux,)
    hqp:  (nh, nh) Hqp, occupied levels first; leading (vt+ct) window used.
    vt, ct: BSE occupied / virtual counts; voff = vmin - rpamin, coff = cmin - rpamin.
    """

    def __init__(self, mmn, w, hqp, vt, ct, voff=0, coff=None):
        self.mmn = np.ascontiguousarray(mmn, dtype=np.float64)
        self.w = np.ascontiguousarray(w, dtype=np.float64)
        self.hqp = np.asfortranarray(hqp, dtype=np.float64)
        self.nm, self.naux, self.nn = self.mmn.shape
        self.vt, self.ct = int(vt), int(ct)
        self.voff = int(voff)
        self.coff = int(self.voff + vt if coff is None else coff)
        self.dim = self.vt * self.ct

    def _common(self, coef):
        return [_p(self.mmn), self.nm, self.nn, self.naux, _p(self.w), _p(self.hqp),
                self.hqp.shape[0], self.vt, self.ct, self.voff, self.coff, *coef]

    def matmul_ref(self, X, op="singlet", c1_range=None, v1_range=None):
        """Reference loop nest (row-built Hd, v-pair Hx)."""
        X = np.asfortranarray(X, dtype=np.float64)
        if X.ndim == 1:
            X = X.reshape(-1, 1, order="F")
        k = X.shape[1]
        Y = np.zeros((self.dim, k), order="F")
        c1 = c1_range or (0, self.ct)
        v1 = v1_range or (0, self.vt)
        lib().oracle_bse_matmul_ref(*self._common(OPERATORS[op]), _p(X), self.dim, k, _p(Y), self.dim,
                                    c1[0], c1[1], v1[0], v1[1])
        return Y

    def matmul_fact(self, X, op="singlet"):
        X = np.asfortranarray(X, dtype=np.float64)
        if X.ndim == 1:
            X = X.reshape(-1, 1, order="F")
        k = X.shape[1]
        Y = np.zeros((self.dim, k), order="F")
        lib().oracle_bse_matmul_fact(*self._common(OPERATORS[op]), _p(X), self.dim, k, _p(Y), self.dim)
        return Y

    def matmul_rows(self, X, rows, op="singlet"):
        """Rows `rows` (pair indices) of H X, each row built as the reference loop nest
        builds it; returns a (len(rows), k) array."""
        X = np.asfortranarray(X, dtype=np.float64)
        if X.ndim == 1:
            X = X.reshape(-1, 1, order="F")
        k = X.shape[1]
        r = np.ascontiguousarray(rows, dtype=np.int64)
        if r.size and (r.min() < 0 or r.max() >= self.dim):
            raise IndexError("matmul_rows: row index outside the operator")
        Y = np.zeros((r.size, k), order="F")
        lib().oracle_bse_matmul_rows(*self._common(OPERATORS[op]), _p(X), self.dim, k,
                                     r.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)), r.size, _p(Y))
        return Y

    def diagonal(self, op="singlet"):
        D = np.zeros(self.dim)
        lib().oracle_bse_diagonal(*self._common(OPERATORS[op]), _p(D))
        return D

    def ham_matmul(self, X, a_op="singlet", b_op="singlet_b", use_ref_loop=True):
        X = np.asfortranarray(X, dtype=np.float64)
        k = X.shape[1]
        Y = np.zeros((2 * self.dim, k), order="F")
        ac = (ctypes.c_int * 4)(*OPERATORS[a_op])
        bc = (ctypes.c_int * 4)(*OPERATORS[b_op])
        lib().oracle_ham_matmul(_p(self.mmn), self.nm, self.nn, self.naux, _p(self.w), _p(self.hqp),
                                self.hqp.shape[0], self.vt, self.ct, self.voff, self.coff, ac, bc,
                                _p(X), k, _p(Y), int(bool(use_ref_loop)))
        return Y

    def dense(self, op="singlet", ref_loop=False):
        eye = np.eye(self.dim, order="F")
        return self.matmul_ref(eye, op) if ref_loop else self.matmul_fact(eye, op)


def set_threads(n):
    lib().oracle_set_threads(int(n))


def num_threads():
    return int(lib().oracle_num_threads())
