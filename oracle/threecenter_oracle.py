"""CPU restatement of the Mmn producer (TEST INFRASTRUCTURE ONLY: tests/ compare against it).

  fill_3c_mo             TCMatrix_gwbse::Fill3cMO (xtp/src/libxtp/libint2_calls.cc:595-651):
                         every aux function P: (dftn A_P) dftm with dftn = C[:, n-window]^T,
                         dftm = C[:, m-window]; block[m](n, P) = result(n, m)
  pseudo_inv_sqrt        AOCoulomb::Pseudo_InvSqrt (xtp/src/libxtp/aomatrices/aomatrix.cc:88-102)
  pseudo_inv_sqrt_gwbse  AOCoulomb::Pseudo_InvSqrt_GWBSE (aomatrix.cc:53-86)

The two metric functions are pinned against the reference's golden matrices
(xtp/src/tests/DataFiles/aomatrix/coulombinvsqrt*_ref.mm, tests/golden/aomatrix.npz).
The transform has no golden data usable here (its test needs libint2 integrals).
"""
from __future__ import annotations

import numpy as np


def fill_3c_mo(ao3c, C, mmin, mmax, nmin, nmax):
    """ao3c: (naux, nbf, nbf) with ao3c[P] the symmetric (P|mu nu) matrix; C: (nbf, nmo).
    Returns (msize, naux, nsize) with M(m, n, P) = out[m - mmin, P, n - nmin]."""
    dftm = C[:, mmin:mmax + 1]
    dftn = C[:, nmin:nmax + 1].T
    naux = ao3c.shape[0]
    out = np.zeros((mmax - mmin + 1, naux, nmax - nmin + 1))
    for P in range(naux):
        r = (dftn @ ao3c[P]) @ dftm          # (nsize x msize)
        out[:, P, :] = r.T
    return out


def _inv_sqrt_weights(lam, etol):
    f = np.zeros_like(lam)
    keep = lam >= etol
    f[keep] = 1.0 / np.sqrt(lam[keep])
    return f, int(np.count_nonzero(~keep))


def pseudo_inv_sqrt(V, etol):
    lam, U = np.linalg.eigh(V)
    f, removed = _inv_sqrt_weights(lam, etol)
    return (U * f) @ U.T, removed


def pseudo_inv_sqrt_gwbse(S, V, etol):
    lo, Uo = np.linalg.eigh(S)
    fo, r1 = _inv_sqrt_weights(lo, etol)
    Ssqrt = (Uo * fo) @ Uo.T
    ortho = Ssqrt @ V @ Ssqrt
    le, Ue = np.linalg.eigh(ortho)
    fe, r2 = _inv_sqrt_weights(le, etol)
    Vm1 = (Ue * fe) @ Ue.T
    return (Vm1 @ Ssqrt).T, r1 + r2
