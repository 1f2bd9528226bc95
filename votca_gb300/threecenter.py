"""Producer side of the Mmn tensor on the GPU, mirroring TCMatrix_gwbse
(xtp/src/libxtp/threecenter.cc, xtp/src/libxtp/libint2_calls.cc) and the auxiliary
Coulomb metric of AOCoulomb (xtp/src/libxtp/aomatrices/aomatrix.cc):

  fill_3c_mo                      TCMatrix_gwbse::Fill3cMO, with the AO three-centre
                                  integrals (P|mu nu) given by the caller (no integral
                                  engine in this library)
  multiply_right_with_aux_matrix  TCMatrix_gwbse::MultiplyRightWithAuxMatrix
  pseudo_inv_sqrt                 AOCoulomb::Pseudo_InvSqrt
  pseudo_inv_sqrt_gwbse           AOCoulomb::Pseudo_InvSqrt_GWBSE
  fill                            TCMatrix_gwbse::Fill: Fill3cMO, then the product with
                                  Pseudo_InvSqrt_GWBSE(aux overlap, 5e-7) of the aux Coulomb
                                  matrix (threecenter.cc:79-95)
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .bse_operator import TCMatrix_gwbse, _p


def _slices(Mmn: TCMatrix_gwbse):
    d = Mmn.data
    desc = _lib.bse_mmn_desc(Mmn.auxsize(), Mmn.get_mmin(), Mmn.get_mmax(), Mmn.get_nmin(), Mmn.get_nmax())
    ptrs = (_lib.c_dp * Mmn.msize())(*[ctypes.cast(d.ctypes.data + m * d.strides[0], _lib.c_dp)
                                       for m in range(Mmn.msize())])
    return desc, ptrs


def fill_3c_mo(Mmn: TCMatrix_gwbse, ao3c, dft_orbitals):
    """Overwrites Mmn with M(m, n, P) = sum_{mu,nu} C(mu, n) (P|mu nu) C(nu, m).
    ao3c: (auxsize, nbf, nbf), ao3c[P] symmetric; dft_orbitals: (nbf, nmo)."""
    L = _lib.load()
    A = np.ascontiguousarray(ao3c, dtype=np.float64)
    C = np.asfortranarray(dft_orbitals, dtype=np.float64)
    naux, nbf = A.shape[0], A.shape[1]
    if A.shape != (naux, nbf, nbf) or naux != Mmn.auxsize() or C.shape[0] != nbf:
        raise _lib.BSEError(1, "fill_3c_mo: ao3c must be (auxsize, nbf, nbf) and dft_orbitals (nbf, nmo)")
    desc, ptrs = _slices(Mmn)
    # slice P of the C-ordered (naux, nbf, nbf) array is the column-major (mu, nu) matrix of
    # its transpose; the matrices are symmetric
    _lib.check(L.bse_mmn_fill_3c_mo(ctypes.byref(desc), ptrs, _p(A), nbf, _p(C), nbf, C.shape[1]))
    return Mmn


def multiply_right_with_aux_matrix(Mmn: TCMatrix_gwbse, U):
    L = _lib.load()
    U = np.asfortranarray(U, dtype=np.float64)
    desc, ptrs = _slices(Mmn)
    _lib.check(L.bse_mmn_multiply_right(ctypes.byref(desc), ptrs, _p(U), U.shape[0]))
    return Mmn


def pseudo_inv_sqrt(V, etol):
    """(V^-1/2 over eigenvalues >= etol, number of removed functions)."""
    L = _lib.load()
    V = np.asfortranarray(V, dtype=np.float64)
    n = V.shape[0]
    out = np.zeros((n, n), order="F")
    removed = ctypes.c_int64()
    _lib.check(L.bse_aux_pseudo_inv_sqrt(n, _p(V), n, etol, _p(out), n, ctypes.byref(removed)))
    return out, removed.value


def pseudo_inv_sqrt_gwbse(S, V, etol):
    """((V'^-1/2 S^-1/2)^T with V' = S^-1/2 V S^-1/2, number of removed functions)."""
    L = _lib.load()
    S = np.asfortranarray(S, dtype=np.float64)
    V = np.asfortranarray(V, dtype=np.float64)
    n = V.shape[0]
    out = np.zeros((n, n), order="F")
    removed = ctypes.c_int64()
    _lib.check(L.bse_aux_pseudo_inv_sqrt_gwbse(n, _p(S), n, _p(V), n, etol, _p(out), n, ctypes.byref(removed)))
    return out, removed.value


def fill(Mmn: TCMatrix_gwbse, ao3c, dft_orbitals, aux_overlap, aux_coulomb, etol=5e-7):
    """TCMatrix_gwbse::Fill; returns the number of removed auxiliary functions."""
    fill_3c_mo(Mmn, ao3c, dft_orbitals)
    inv_sqrt, removed = pseudo_inv_sqrt_gwbse(aux_overlap, aux_coulomb, etol)
    multiply_right_with_aux_matrix(Mmn, inv_sqrt)
    return removed
