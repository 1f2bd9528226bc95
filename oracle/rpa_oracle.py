"""NumPy restatement of the static screening that feeds Hd (TEST INFRASTRUCTURE ONLY).

  epsilon_r        RPA::calculate_epsilon_r, xtp/src/libxtp/gwbse/rpa.cc:145-200
                   (eta = 1e-4 as RPA::eta_, xtp/include/votca/xtp/rpa.h:90)
  setup_screening  BSE::SetupDirectInteractionOperator, xtp/src/libxtp/gwbse/bse.cc:188-204:
                   eigen-decompose eps, rotate Mmn by its eigenvectors
                   (MultiplyRightWithAuxMatrix, threecenter.cc:54-65), epsilon_0_inv = 1/lambda
                   for lambda > 1e-8
"""
import numpy as np

ETA = 1e-4


def epsilon_r(mmn, energies, homo, rpamin, rpamax, freq=0.0 + 0.0j, mmin=0):
    """mmn: (msize, naux, nsize) reference slice layout, slice index = level - mmin."""
    naux = mmn.shape[1]
    lumo = homo + 1
    n_occ = lumo - rpamin
    n_unocc = rpamax - lumo + 1
    res = np.zeros((naux, naux))
    for m in range(n_occ):
        M = mmn[rpamin + m - mmin][:, -n_unocc:].T          # bottomRows(n_unocc): (n_unocc, naux)
        dE = energies[-n_unocc:] - energies[m]
        dm = freq.real - dE
        dp = freq.real + dE
        chi = dm / (dm**2 + (freq.imag + ETA) ** 2) - dp / (dp**2 + (freq.imag - ETA) ** 2)
        res += M.T @ (chi[:, None] * M)
    return np.eye(naux) - 2.0 * res


def setup_screening(mmn, eps):
    lam, U = np.linalg.eigh(eps)
    rotated = np.einsum("mpn,pq->mqn", mmn, U)
    w = np.where(lam > 1e-8, 1.0 / np.where(lam > 1e-8, lam, 1.0), 0.0)
    return rotated, w
