"""Transition dipoles and oscillator strengths of BSE states (TEST INFRASTRUCTURE ONLY).

Only tests/ use this module, as the reference of bse_transition_dipoles.  It restates
  Orbitals::CalcFreeTransition_Dipoles    xtp/src/libxtp/orbitals.cc:740-757
      interlevel dipoles D_i = C_virt^T dip_i C_occ (ctotal x vtotal)
  Orbitals::CalcCoupledTransition_Dipoles  orbitals.cc:763-800 (restricted singlets: the
      state's coefficients (X + Y for full BSE) mapped as a ctotal x vtotal matrix, summed
      against D_i, times -sqrt(2)) and :804-877 (combined UKS excitons: both spin blocks,
      times -1)
  Orbitals::Oscillatorstrengths            orbitals.cc:645-673 (f = 2/3 Omega |d|^2)
The map takes the leading vtotal * ctotal entries of each state's vector, as Eigen::Map does.
"""
from __future__ import annotations

import numpy as np


def interlevel_dipoles(ao_dip, C, vmin, vtotal, cmin, ctotal):
    occ = C[:, vmin:vmin + vtotal]
    virt = C[:, cmin:cmin + ctotal]
    return [virt.T @ ao_dip[i] @ occ for i in range(3)]


def transition_dipoles(ao_dip, C, vmin, vtotal, cmin, ctotal, X, Y=None, prefactor=-np.sqrt(2.0)):
    """(nstates, 3) transition dipoles of one spin block."""
    D = interlevel_dipoles(ao_dip, C, vmin, vtotal, cmin, ctotal)
    X = np.asarray(X, dtype=np.float64)
    coeffs = X + (np.asarray(Y, dtype=np.float64) if Y is not None else 0.0)
    out = np.zeros((coeffs.shape[1], 3))
    for s in range(coeffs.shape[1]):
        mat = coeffs[:vtotal * ctotal, s].reshape((ctotal, vtotal), order="F")
        for i in range(3):
            out[s, i] = prefactor * float(np.sum(mat * D[i]))
    return out


def oscillator_strengths(omega, dipoles):
    return np.sum(np.asarray(dipoles) ** 2, axis=1) * 2.0 / 3.0 * np.asarray(omega)
