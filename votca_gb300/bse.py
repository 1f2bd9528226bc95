"""Mirror of the BSE solve drivers of VOTCA-XTP (xtp/src/libxtp/gwbse/bse.cc).

  adjust_hqp_size             BSE::AdjustHqpSize, bse.cc:147-186 (and BSE::configure's
                              diagonal-only choice, bse.cc:53-57; per spin channel it is
                              BSE_UKS::AdjustHqpSize, bse_uks.cc:92-133)
  solve_hermitian             BSE::solve_hermitian, bse.cc:266-293
  solve_nonhermitian_davidson BSE::Solve_nonhermitian_Davidson, bse.cc:315-360
  full_bse_ranked_guess       BuildFullBSEXRankedInitialGuess,
                              xtp/include/votca/xtp/bse_initialization.h:47-92
  exciton_weights             the transitions BSE::Analyze_singlets / Analyze_triplets print
                              per root (PrintWeights, bse.cc:378-391), as data
  expectation_value_operator  BSE::ExpectationValue_Operator, bse.cc:500-520
  analyze_eh_interaction      BSE::Analyze_eh_interaction, bse.cc:551-606 (with
                              ExchangePrefactor, bse.cc:136-145)

The Davidson iteration itself runs on the GPU (bse_davidson_solve).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .bse_operator import HamiltonianOperator, HdOperator, Hd2Operator, HqpOperator, HxOperator
from .davidson import DavidsonSolver


@dataclass
class DavidsonOptions:
    """The BSE Davidson knobs of xtp/share/xtp/xml/subpackages/gwbse.xml."""
    davidson_correction: str = "DPR"
    davidson_tolerance: object = "normal"  # preset name or a number
    davidson_update: str = "safe"
    davidson_maxiter: int = 50
    nmax: int = 5
    # no counterpart in gwbse.xml: trial vectors per iteration (0 = the davidson_update rule)
    # and the FP64 polish of split-precision solves
    davidson_block: int = 0
    fp64_polish: object = True  # True / "sliced", "fp64" (FP64 DGEMM products) or False


def adjust_hqp_size(Hqp, rpa_input_energies, homo, vmin, cmax, qpmin, qpmax, rpamin,
                    use_hqp_offdiag=False):
    """The (vtotal + ctotal)^2 Hqp window the operator reads (occupied first): the QP
    Hamiltonian (qpmin..qpmax) where the BSE window overlaps it, and the RPA input energies
    (indexed from rpamin) on the diagonal of the levels outside the QP range.  Without
    use_hqp_offdiag only the diagonal is kept."""
    Hqp = np.asarray(Hqp, dtype=np.float64)
    e = np.asarray(rpa_input_energies, dtype=np.float64)
    vtotal, ctotal = homo - vmin + 1, cmax - homo
    n = vtotal + ctotal
    gwsize = qpmax - qpmin + 1
    rpa_off = vmin - rpamin
    if Hqp.shape != (gwsize, gwsize):
        raise ValueError("adjust_hqp_size: Hqp must be (qpmax - qpmin + 1) square")
    out = np.zeros((n, n))
    if vmin >= qpmin:
        start = vmin - qpmin
        if cmax <= qpmax:
            out[:, :] = Hqp[start:start + n, start:start + n]
        else:
            virt = gwsize - start
            out[:virt, :virt] = Hqp[start:start + virt, start:start + virt]
            extra = cmax - qpmax
            out[np.arange(n - extra, n), np.arange(n - extra, n)] = e[rpa_off + virt:rpa_off + virt + extra]
    else:
        occ = qpmin - vmin
        if occ + gwsize > n:
            raise ValueError("adjust_hqp_size: the QP range extends beyond the BSE window")
        out[np.arange(occ), np.arange(occ)] = e[rpa_off:rpa_off + occ]
        out[occ:occ + gwsize, occ:occ + gwsize] = Hqp
        if cmax > qpmax:
            virt = occ + gwsize
            extra = cmax - qpmax
            out[np.arange(n - extra, n), np.arange(n - extra, n)] = e[rpa_off + virt:rpa_off + virt + extra]
    return out if use_hqp_offdiag else np.diag(np.diag(out))


def _solver(opt: DavidsonOptions):
    ds = DavidsonSolver()
    ds.set_correction(opt.davidson_correction)
    ds.set_tolerance(opt.davidson_tolerance)
    ds.set_size_update(opt.davidson_update)
    ds.set_iter_max(opt.davidson_maxiter)
    ds.set_max_search_space(10 * opt.nmax)
    ds.set_block_size(opt.davidson_block)
    ds.set_fp64_polish(opt.fp64_polish)
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


def _expval(a, b):
    return np.sum(a * b, axis=0)


def expectation_value_operator(H, X, Y=None):
    """(direct, cross) of operator H for eigenvectors X (and Y for full BSE): direct = X.HX
    (+ Y.HY), cross = 2 Y.HX (empty in TDA).  One product per block on the GPU."""
    X = np.asfortranarray(X, dtype=np.float64)
    HX = H.matmul(X)
    direct = _expval(X, HX)
    if Y is None:
        return direct, np.zeros(0)
    Y = np.asfortranarray(Y, dtype=np.float64)
    direct = direct + _expval(Y, H.matmul(Y))
    return direct, 2.0 * _expval(Y, HX)


def exchange_prefactor(spin):
    if spin == "singlet":
        return 2.0
    if spin == "triplet":
        return 0.0
    raise RuntimeError("Unsupported QMStateType in BSE::ExchangePrefactor")


def analyze_eh_interaction(ctx, X, Y=None, spin="singlet"):
    """Composition of the excitation energies (per root): qp_contrib = <Hqp>, direct_contrib =
    <-Hd> (+ the 2 Y.(-Hd2)X cross term in full BSE), exchange_contrib = eta <Hx> (+ its
    cross term), eta = 2 for singlets, 0 for triplets.  For normalised eigenpairs the three
    add up to the excitation energy."""
    out = {"qp_contrib": expectation_value_operator(HqpOperator(ctx), X, Y)[0]}
    direct, _ = expectation_value_operator(HdOperator(ctx), X, Y)
    if Y is not None:
        direct = direct + expectation_value_operator(Hd2Operator(ctx), X, Y)[1]
    out["direct_contrib"] = direct
    xpref = exchange_prefactor(spin)
    if xpref != 0.0:
        d, cr = expectation_value_operator(HxOperator(ctx), X, Y)
        out["exchange_contrib"] = xpref * (d + cr if Y is not None else d)
    else:
        out["exchange_contrib"] = np.zeros(direct.size)
    return out


def exciton_weights(homo, vmin, cmax, X, Y=None, min_print_weight=0.5):
    """Per root, the pairs whose weight |X|^2 (TDA) or |X|^2 - |Y|^2 (full BSE) exceeds
    min_print_weight (the gwbse option print_weight, default 0.5), in pair order, as
    (HOMO-i, LUMO+j, weight) with i = homo - v and j = c - homo - 1 (vc2index levels
    v = vmin + I // ctotal, c = homo + 1 + I % ctotal)."""
    X = np.asarray(X, dtype=np.float64)
    if X.ndim == 1:
        X = X[:, None]
    w = X * X
    if Y is not None:
        Yv = np.asarray(Y, dtype=np.float64).reshape(X.shape)
        w = w - Yv * Yv
    ctotal = cmax - homo
    if X.shape[0] != (homo - vmin + 1) * ctotal:
        raise ValueError("exciton_weights: vectors do not match the BSE window")
    out = []
    for k in range(X.shape[1]):
        rows = []
        for i in np.nonzero(w[:, k] > min_print_weight)[0]:
            v, c = vmin + i // ctotal, homo + 1 + i % ctotal
            rows.append((int(homo - v), int(c - homo - 1), float(w[i, k])))
        out.append(rows)
    return out
