"""Host-side mirror of VOTCA-XTP's BSE operator interface, backed by the GPU.

Names, argument meaning and error behaviour follow the reference:
  BSEOperator_Options                     xtp/include/votca/xtp/bse_operator.h:32-38
  BSE_OPERATOR<cqp,cx,cd,cd2>             bse_operator.h:40-76 (matmul, diagonal, rows/cols)
  SingletOperator_TDA ... Hd2Operator     bse_operator.h:79-87
  TCMatrix_gwbse (Mmn container)          xtp/include/votca/xtp/threecenter.h:70-142
  HamiltonianOperator<A, B>               xtp/include/votca/xtp/bseoperator_btda.h:44-149

All arithmetic runs on the device through the C ABI (libvotca_gb300.so); this
module only marshals arrays.  Errors raise BSEError (a RuntimeError, as the
reference throws std::runtime_error).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib

PRECISION_FP64 = 0
PRECISION_MIXED = 1
PRECISION_SLICED = 2


@dataclass
class BSEOperator_Options:
    homo: int
    rpamin: int
    qpmin: int
    vmin: int
    cmax: int


class TCMatrix_gwbse:
    """Mmn three-centre MO tensor: msize() slices, slice m a [nsize x auxsize] matrix.

    Stored as a (msize, auxsize, nsize) C-contiguous array, which is exactly the
    reference's vector of column-major [nsize x auxsize] slices laid end to end:
    M(m, n, P) = data[m - mmin, P, n - nmin].
    """

    def __init__(self, data, mmin=0, nmin=0):
        self.data = np.ascontiguousarray(data, dtype=np.float64)
        self.mmin_ = int(mmin)
        self.nmin_ = int(nmin)

    @classmethod
    def Initialize(cls, basissize, mmin, mmax, nmin, nmax):
        return cls(np.zeros((mmax - mmin + 1, basissize, nmax - nmin + 1)), mmin, nmin)

    def auxsize(self):
        return self.data.shape[1]

    def msize(self):
        return self.data.shape[0]

    def nsize(self):
        return self.data.shape[2]

    def get_mmin(self):
        return self.mmin_

    def get_mmax(self):
        return self.mmin_ + self.msize() - 1

    def get_nmin(self):
        return self.nmin_

    def get_nmax(self):
        return self.nmin_ + self.nsize() - 1

    def __getitem__(self, m):
        """Slice m as an (nsize x auxsize) view, like Mmn_[m]."""
        return self.data[m].T


def _p(a):
    return a.ctypes.data_as(_lib.c_dp)


class GpuBSEContext:
    """Device-resident staging of (epsilon_0_inv or dense W, Mmn, Hqp) for one
    BSE window.  Several BSE_OPERATOR coefficient sets share one context."""

    def __init__(self, epsilon_0_inv, Mmn: TCMatrix_gwbse, Hqp, opt: BSEOperator_Options,
                 precision=PRECISION_FP64, dense_screening=None):
        L = _lib.load()
        self._L = L
        desc = _lib.bse_mmn_desc(Mmn.auxsize(), Mmn.get_mmin(), Mmn.get_mmax(), Mmn.get_nmin(), Mmn.get_nmax())
        ptrs = (_lib.c_dp * Mmn.msize())(*[
            ctypes.cast(Mmn.data.ctypes.data + m * Mmn.data.strides[0], _lib.c_dp) for m in range(Mmn.msize())])
        hqp = np.asfortranarray(Hqp, dtype=np.float64)
        o = _lib.bse_options(opt.homo, opt.rpamin, opt.qpmin, opt.vmin, opt.cmax)
        h = ctypes.c_void_p()
        if dense_screening is not None:
            W = np.asfortranarray(dense_screening, dtype=np.float64)
            _lib.check(L.bse_op_create_dense_screening(ctypes.byref(desc), ptrs, _p(W), _p(hqp), hqp.shape[0],
                                                       hqp.shape[0], ctypes.byref(o), precision, ctypes.byref(h)))
        else:
            if epsilon_0_inv is None:
                raise _lib.BSEError(1, "GpuBSEContext: epsilon_0_inv or dense_screening is required")
            w = np.ascontiguousarray(epsilon_0_inv, dtype=np.float64)
            _lib.check(L.bse_op_create(ctypes.byref(desc), ptrs, _p(w), _p(hqp), hqp.shape[0], hqp.shape[0],
                                       ctypes.byref(o), precision, ctypes.byref(h)))
        self.handle = h
        n = ctypes.c_int64()
        _lib.check(L.bse_op_size(h, ctypes.byref(n)))
        self.size = n.value
        self.opt = opt
        self.precision = precision

    def close(self):
        if self.handle:
            _lib.check(self._L.bse_op_destroy(self.handle))
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DenseGpuOperator:
    """A dense symmetric matrix as a device operator (the reference tests'
    HermitianBlockOperator); with b given, HAM products use [[a, b], [-b, -a]]."""

    def __init__(self, a, b=None):
        L = _lib.load()
        self._L = L
        a = np.asfortranarray(a, dtype=np.float64)
        bb = None if b is None else np.asfortranarray(b, dtype=np.float64)
        h = ctypes.c_void_p()
        _lib.check(L.bse_dense_op_create(_p(a), None if bb is None else _p(bb), a.shape[0], a.shape[0],
                                         ctypes.byref(h)))
        self.handle = h
        self.size = a.shape[0]
        self.coef = (0, 0, 0, 0)
        self.has_b = b is not None

    def rows(self):
        return self.size

    def cols(self):
        return self.size

    def matmul(self, X):
        return _matmul(self._L, self.handle, (0, 0, 0, 0), X, self.size)

    def diagonal(self):
        D = np.zeros(self.size)
        _lib.check(self._L.bse_op_diagonal(self.handle, 0, 0, 0, 0, _p(D)))
        return D

    def __matmul__(self, X):
        return self.matmul(X)

    def close(self):
        if self.handle:
            _lib.check(self._L.bse_op_destroy(self.handle))
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _matmul(L, handle, coef, X, size):
    X = np.asfortranarray(X, dtype=np.float64)
    squeeze = X.ndim == 1
    if squeeze:
        X = X.reshape(-1, 1, order="F")
    if X.shape[0] != size:
        raise _lib.BSEError(1, f"matmul: input has {X.shape[0]} rows, operator size is {size}")
    k = X.shape[1]
    Y = np.zeros((size, k), order="F")
    _lib.check(L.bse_op_matmul(handle, *coef, _p(X), size, k, _p(Y), size))
    return Y[:, 0] if squeeze else Y


class BSE_OPERATOR:
    """BSE_OPERATOR<cqp, cx, cd, cd2> on a GpuBSEContext: applies
    cqp*Hqp + cx*Hx - cd*Hd - cd2*Hd2."""

    cqp = cx = cd = cd2 = 0

    def __init__(self, ctx: GpuBSEContext, cqp=None, cx=None, cd=None, cd2=None):
        if cqp is not None:
            self.cqp, self.cx, self.cd, self.cd2 = cqp, cx, cd, cd2
        if self.cd != 0 and self.cd2 != 0:
            raise _lib.BSEError(1, "Hamiltonian cannot contain Hd and Hd2 at the same time")
        self.ctx = ctx

    @property
    def coef(self):
        return (self.cqp, self.cx, self.cd, self.cd2)

    def rows(self):
        return self.ctx.size

    def cols(self):
        return self.ctx.size

    def size(self):
        return self.ctx.size

    def matmul(self, X):
        return _matmul(self.ctx._L, self.ctx.handle, self.coef, X, self.ctx.size)

    def __matmul__(self, X):
        return self.matmul(X)

    def diagonal(self):
        D = np.zeros(self.ctx.size)
        _lib.check(self.ctx._L.bse_op_diagonal(self.ctx.handle, *self.coef, _p(D)))
        return D

    def matmul_device(self, dX_ptr, ldx, k, dY_ptr, ldy, stream=0):
        """Device-pointer product (pointers as ints), stream-ordered on `stream`."""
        _lib.check(self.ctx._L.bse_op_matmul_device(self.ctx.handle, *self.coef, ctypes.c_void_p(dX_ptr), ldx, k,
                                                    ctypes.c_void_p(dY_ptr), ldy, ctypes.c_void_p(stream)))


def _preset(name, c):
    return type(name, (BSE_OPERATOR,), {"cqp": c[0], "cx": c[1], "cd": c[2], "cd2": c[3]})


SingletOperator_TDA = _preset("SingletOperator_TDA", (1, 2, 1, 0))
TripletOperator_TDA = _preset("TripletOperator_TDA", (1, 0, 1, 0))
SingletOperator_BTDA_B = _preset("SingletOperator_BTDA_B", (0, 2, 0, 1))
HqpOperator = _preset("HqpOperator", (1, 0, 0, 0))
HxOperator = _preset("HxOperator", (0, 1, 0, 0))
HdOperator = _preset("HdOperator", (0, 0, 1, 0))
Hd2Operator = _preset("Hd2Operator", (0, 0, 0, 1))


class HamiltonianOperator:
    """[[A, B], [-B, -A]] for two BSE_OPERATORs on the same context (or a dense
    operator holding both blocks)."""

    def __init__(self, A, B):
        self.A_, self.B_ = A, B
        self._size = 2 * A.cols()

    def rows(self):
        return self._size

    def cols(self):
        return self._size

    def diagonal(self):
        d = self.A_.diagonal()
        return np.concatenate([d, -d])

    def matmul(self, X):
        X = np.asfortranarray(X, dtype=np.float64)
        if X.shape[0] != self._size:
            raise _lib.BSEError(1, "HamiltonianOperator: wrong number of rows")
        k = X.shape[1]
        Y = np.zeros((self._size, k), order="F")
        if isinstance(self.A_, DenseGpuOperator):
            L, h = self.A_._L, self.A_.handle
            a = b = (ctypes.c_int32 * 4)(0, 0, 0, 0)
        else:
            L, h = self.A_.ctx._L, self.A_.ctx.handle
            if self.B_.ctx is not self.A_.ctx:
                raise _lib.BSEError(1, "HamiltonianOperator: A and B must share a context")
            a = (ctypes.c_int32 * 4)(*self.A_.coef)
            b = (ctypes.c_int32 * 4)(*self.B_.coef)
        _lib.check(L.bse_ham_matmul(h, a, b, _p(X), self._size, k, _p(Y), self._size))
        return Y

    def __matmul__(self, X):
        return self.matmul(X)
