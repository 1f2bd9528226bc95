"""Screening that feeds the direct term, and the perturbative dynamical screening of
the excitation energies, on the GPU.

  update_rpa_input_energies    RPA::UpdateRPAInputEnergies / ShiftUncorrectedEnergies
                               (rpa.cc:32-73): the RPA input energies from DFT and QP levels
                               (host arithmetic); update_rpa_input_energies_uks the same per
                               spin channel (rpa_uks.cc:41-71, 163-201)
  rpa_epsilon                  RPA::calculate_epsilon_r (xtp/src/libxtp/gwbse/rpa.cc),
                               bse_rpa_epsilon
  cholesky_inverse             the inverse of a symmetric positive definite matrix,
                               bse_cholesky_inverse (blocked Cholesky on the device)
  positive_inverse             U diag(1/lambda, lambda > cutoff) U^T, bse_positive_inverse
  screened_context             BSE::SetupDirectInteractionOperator (bse.cc:188-204) in the
                               dense form: W = eps(omega)^-1 folded into the operator
  perturbative_dynamical_screening
                               BSE::Perturbative_DynamicalScreening (bse.cc:610-681)
  rpa_epsilon_uks              RPA_UKS::calculate_epsilon_r (rpa_uks.cc:306-358):
                               eps = 1 - R_alpha - R_beta, each channel's sum as in the
                               restricted kernel (which forms 1 - 2 R)
  screened_context_uks         BSE_UKS::SetupDirectInteractionOperator (bse_uks.cc:135-157)
                               in the dense form, on the unrotated (raw) Mmn of both channels
  perturbative_dynamical_screening_uks
                               BSE_UKS::Perturbative_DynamicalScreening (bse_uks.cc:640-715)

The reference diagonalises eps, rotates Mmn by its eigenvectors and weights the rotated
aux functions by 1/lambda (lambda > 1e-8).  With all eigenvalues above that cutoff this is
the same operator as sum_PQ M^P (eps^-1)_PQ M^Q, which is what the dense form computes (by
a Cholesky inverse on the device).  When eps(omega) is not positive definite (omega beyond
the first RPA pole) the modes with lambda <= 1e-8 are dropped as in the reference
(positive_inverse).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .bse_operator import GpuBSEContext, HdOperator, Hd2Operator, TCMatrix_gwbse, _p
from .bse import expectation_value_operator


def _desc_ptrs(Mmn: TCMatrix_gwbse):
    d = Mmn.data
    desc = _lib.bse_mmn_desc(Mmn.auxsize(), Mmn.get_mmin(), Mmn.get_mmax(), Mmn.get_nmin(), Mmn.get_nmax())
    ptrs = (_lib.c_dp * Mmn.msize())(*[ctypes.cast(d.ctypes.data + m * d.strides[0], _lib.c_dp)
                                       for m in range(Mmn.msize())])
    return desc, ptrs


def _rpa_input_energies(dft, gw, qpmin, homo, rpamin, rpamax, absolute_rpa_index):
    dft = np.asarray(dft, dtype=np.float64)
    gw = np.asarray(gw, dtype=np.float64)
    rpatotal = rpamax - rpamin + 1
    gwsize = gw.size
    if rpamin < 0 or rpamax >= dft.size or rpatotal <= 0:
        raise ValueError("update_rpa_input_energies: rpa window outside the DFT levels")
    if qpmin < rpamin or qpmin - rpamin + gwsize > rpatotal:
        raise ValueError("update_rpa_input_energies: QP levels outside the rpa window")
    e = dft[rpamin:rpamax + 1].copy()
    e[qpmin - rpamin:qpmin - rpamin + gwsize] = gw
    qpmax = qpmin + gwsize - 1
    # RPA::getMaxCorrection reads the RPA vector at the absolute level index and the DFT vector
    # at index - rpamin; RPA_UKS::getMaxCorrection the other way round
    ro, do = (0, -rpamin) if absolute_rpa_index else (-rpamin, 0)

    def max_correction(lo, hi):
        n = hi - lo + 1
        if n <= 0:
            return 0.0
        if lo + ro < 0 or lo + ro + n > rpatotal or lo + do < 0 or lo + do + n > dft.size:
            raise ValueError("update_rpa_input_energies: correction range outside the levels")
        return float(np.max(np.abs(e[lo + ro:lo + ro + n] - dft[lo + do:lo + do + n])))

    occ = max_correction(qpmin, homo)
    virt = max_correction(homo + 1, qpmax)
    e[:qpmin if absolute_rpa_index else qpmin - rpamin] -= occ
    tail = rpamax - qpmax
    if tail > 0:
        e[rpatotal - tail:] += virt
    return e


def update_rpa_input_energies(dftenergies, gwaenergies, qpmin, homo, rpamin, rpamax):
    """The energies eps(omega) is built from (rpamin..rpamax): DFT levels with the QP levels
    (qpmin..qpmin + len(gwaenergies) - 1) put in, the levels below qpmin shifted down by the
    largest |QP - DFT| correction among qpmin..homo and those above qpmax shifted up by the
    largest among lumo..qpmax.  Index arithmetic as in RPA::UpdateRPAInputEnergies: the
    corrections read the RPA vector at the absolute level index and the DFT vector at
    index - rpamin, and the lower shift covers the first qpmin entries of the RPA vector (the
    same as the unrestricted form for rpamin = 0, the GW-BSE default).  An empty correction
    range contributes 0."""
    return _rpa_input_energies(dftenergies, gwaenergies, qpmin, homo, rpamin, rpamax, True)


def update_rpa_input_energies_uks(dft_alpha, dft_beta, gw_alpha, gw_beta, qpmin, homo_alpha, homo_beta,
                                  rpamin, rpamax):
    """RPA_UKS::UpdateRPAInputEnergies (rpa_uks.cc:41-71, 163-201): the restricted recipe per
    spin channel with its own HOMO, indexing the RPA vector from rpamin throughout.
    Returns (energies_alpha, energies_beta)."""
    return (_rpa_input_energies(dft_alpha, gw_alpha, qpmin, homo_alpha, rpamin, rpamax, False),
            _rpa_input_energies(dft_beta, gw_beta, qpmin, homo_beta, rpamin, rpamax, False))


def rpa_epsilon(Mmn: TCMatrix_gwbse, rpa_energies, homo, rpamin, rpamax, frequency=0.0):
    """eps(omega) (auxsize x auxsize) of the RPA on the levels rpamin..rpamax."""
    L = _lib.load()
    e = np.ascontiguousarray(rpa_energies, dtype=np.float64)
    naux = Mmn.auxsize()
    eps = np.zeros((naux, naux), order="F")
    desc, ptrs = _desc_ptrs(Mmn)
    w = complex(frequency)
    _lib.check(L.bse_rpa_epsilon(ctypes.byref(desc), ptrs, _p(e), e.size, homo, rpamin, rpamax, w.real, w.imag,
                                 _p(eps)))
    return eps


def cholesky_inverse(A):
    L = _lib.load()
    A = np.asfortranarray(A, dtype=np.float64)
    n = A.shape[0]
    Ai = np.zeros((n, n), order="F")
    _lib.check(L.bse_cholesky_inverse(n, _p(A), n, _p(Ai), n))
    return Ai


def positive_inverse(A, cutoff=1e-8):
    """U diag(w) U^T with w = 1/lambda for eigenvalues lambda > cutoff, else 0."""
    L = _lib.load()
    A = np.asfortranarray(A, dtype=np.float64)
    n = A.shape[0]
    W = np.zeros((n, n), order="F")
    _lib.check(L.bse_positive_inverse(n, _p(A), n, cutoff, _p(W), n))
    return W


def screened_context(Mmn, Hqp, opt, rpa_energies, rpa_window, frequency=0.0, precision=0):
    """Operator context with the direct term screened as SetupDirectInteractionOperator
    screens it at `frequency`: eps^-1 by Cholesky when eps is positive definite, else the
    eigenmodes with lambda > 1e-8 only (the reference's cutoff)."""
    homo, rpamin, rpamax = rpa_window
    eps = rpa_epsilon(Mmn, rpa_energies, homo, rpamin, rpamax, frequency)
    try:
        W = cholesky_inverse(eps)
    except _lib.BSEError as e:
        if e.code != 5:  # BSE_ERR_NUMERICAL: not positive definite
            raise
        W = positive_inverse(eps, 1e-8)
    return GpuBSEContext(None, Mmn, Hqp, opt, precision=precision, dense_screening=W)


def _direct(ctx, X, Y):
    direct, _ = expectation_value_operator(HdOperator(ctx), X, Y)
    if Y is not None:
        direct = direct + expectation_value_operator(Hd2Operator(ctx), X, Y)[1]
    return direct


def perturbative_dynamical_screening(Mmn, Hqp, opt, rpa_energies, rpa_window, energies, X, Y=None,
                                     max_iter=10, tolerance=1e-5, precision=0):
    """Excitation energies with the direct term screened at the excitation's own energy,
    to first order around the static solution (energies, X[, Y]) of the same operator:
    Omega_i <- Omega_i + <-Hd(0)>_i - <-Hd(Omega_i')>_i, iterated on Omega_i' until two
    successive values differ by less than `tolerance` or `max_iter` rounds are done."""
    energies = np.asarray(energies, dtype=np.float64)
    X = np.asfortranarray(X, dtype=np.float64)
    Y = None if Y is None else np.asfortranarray(Y, dtype=np.float64)
    static = screened_context(Mmn, Hqp, opt, rpa_energies, rpa_window, 0.0, precision)
    hd_static = _direct(static, X, Y)
    static.close()
    dynamic = energies.copy()
    for i in range(energies.size):
        xi = X[:, i:i + 1]
        yi = None if Y is None else Y[:, i:i + 1]
        for _ in range(max_iter):
            old = dynamic[i]
            ctx = screened_context(Mmn, Hqp, opt, rpa_energies, rpa_window, old, precision)
            hd_dyn = _direct(ctx, xi, yi)[0]
            ctx.close()
            dynamic[i] = energies[i] + hd_static[i] - hd_dyn
            if abs(dynamic[i] - old) < tolerance:
                break
    return dynamic


def rpa_epsilon_uks(Mmn, rpa_energies_alpha, rpa_energies_beta, homo_alpha, homo_beta, rpamin, rpamax,
                    frequency=0.0):
    """eps(omega) of the unrestricted RPA: 1 - R_alpha - R_beta.  The restricted kernel gives
    1 - 2 R_s per channel, so eps = (eps_alpha + eps_beta) / 2."""
    ea = rpa_epsilon(Mmn.alpha, rpa_energies_alpha, homo_alpha, rpamin, rpamax, frequency)
    eb = rpa_epsilon(Mmn.beta, rpa_energies_beta, homo_beta, rpamin, rpamax, frequency)
    return 0.5 * (ea + eb)


def _screening_from(eps):
    try:
        return cholesky_inverse(eps)
    except _lib.BSEError as e:
        if e.code != 5:  # BSE_ERR_NUMERICAL: not positive definite
            raise
        return positive_inverse(eps, 1e-8)


def screened_context_uks(Mmn, Hqp_alpha, Hqp_beta, opt, rpa_energies_alpha, rpa_energies_beta, rpamax,
                         frequency=0.0, precision=0):
    """UKS operator context with the direct terms screened at `frequency` (eps of both
    channels from the raw Mmn, as the reference resets Mmn before each rotation)."""
    from .bse_operator_uks import GpuBSEContextUKS

    eps = rpa_epsilon_uks(Mmn, rpa_energies_alpha, rpa_energies_beta, opt.homo_alpha, opt.homo_beta, opt.rpamin,
                          rpamax, frequency)
    return GpuBSEContextUKS(None, Mmn, Hqp_alpha, Hqp_beta, opt, precision=precision,
                            dense_screening=_screening_from(eps))


def perturbative_dynamical_screening_uks(Mmn, Hqp_alpha, Hqp_beta, opt, rpa_energies_alpha, rpa_energies_beta,
                                         rpamax, energies, X, Y=None, max_iter=10, tolerance=1e-5,
                                         precision=0):
    """UKS excitation energies with the direct terms screened at each excitation's own energy,
    to first order around the static solution (energies, X[, Y]) of the combined operator."""
    from .bse_operator_uks import Hd2UKSOperator, HdUKSOperator

    energies = np.asarray(energies, dtype=np.float64)
    X = np.asfortranarray(X, dtype=np.float64)
    Y = None if Y is None else np.asfortranarray(Y, dtype=np.float64)

    def direct(ctx, x, y):
        d, _ = expectation_value_operator(HdUKSOperator(ctx), x, y)
        if y is not None:
            d = d + expectation_value_operator(Hd2UKSOperator(ctx), x, y)[1]
        return d

    args = (Mmn, Hqp_alpha, Hqp_beta, opt, rpa_energies_alpha, rpa_energies_beta, rpamax)
    static = screened_context_uks(*args, 0.0, precision)
    hd_static = direct(static, X, Y)
    static.close()
    dynamic = energies.copy()
    for i in range(energies.size):
        xi = X[:, i:i + 1]
        yi = None if Y is None else Y[:, i:i + 1]
        for _ in range(max_iter):
            old = dynamic[i]
            ctx = screened_context_uks(*args, old, precision)
            hd_dyn = direct(ctx, xi, yi)[0]
            ctx.close()
            dynamic[i] = energies[i] + hd_static[i] - hd_dyn
            if abs(dynamic[i] - old) < tolerance:
                break
    return dynamic
