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
  transition_dipoles          Orbitals::CalcCoupledTransition_Dipoles, orbitals.cc:740-877
                              (restricted singlets; transition_dipoles_uks for UKS excitons),
                              with caller-supplied AO dipole matrices; on the GPU
  oscillator_strengths        Orbitals::Oscillatorstrengths, orbitals.cc:645-673

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


def _transition_dipoles_block(ao_dipoles, mos, vmin, vtotal, cmin, ctotal, X, Y, prefactor, out, accumulate):
    import ctypes

    from . import _lib

    L = _lib.load()
    A = np.ascontiguousarray(ao_dipoles, dtype=np.float64)
    C = np.asfortranarray(mos, dtype=np.float64)
    Xf = np.asfortranarray(X, dtype=np.float64)
    Yf = None if Y is None else np.asfortranarray(Y, dtype=np.float64)
    nbf = C.shape[0]
    if A.shape != (3, nbf, nbf):
        raise ValueError("transition_dipoles: ao_dipoles must be (3, nbf, nbf) with nbf = mos.shape[0]")
    if Xf.shape[0] < vtotal * ctotal or (Yf is not None and Yf.shape != Xf.shape):
        raise ValueError("transition_dipoles: state vectors shorter than the BSE window")
    # each (nbf x nbf) dipole matrix column-major, the three back to back
    Af = np.ascontiguousarray(np.transpose(A, (0, 2, 1)))
    p = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    _lib.check(L.bse_transition_dipoles(p(Af), nbf, p(C), nbf, C.shape[1], vmin, vtotal, cmin, ctotal, p(Xf),
                                        None if Yf is None else p(Yf), Xf.shape[0], Xf.shape[1], prefactor,
                                        1 if accumulate else 0, p(out)))


def transition_dipoles(ao_dipoles, mos, homo, vmin, cmax, X, Y=None):
    """Transition dipoles (nstates x 3) of restricted BSE singlets: the interlevel dipoles
    C_c^T dip_i C_v (CalcFreeTransition_Dipoles, orbitals.cc:740-757) contracted with each
    state's coefficients (X + Y for full BSE; the leading vtotal * ctotal entries of each column,
    as Eigen::Map reads them) times -sqrt(2) (orbitals.cc:763-800).  ao_dipoles: (3, nbf, nbf)
    AODipole matrices about the caller's origin; mos: (nbf, nmo) MO coefficients."""
    X = np.asarray(X, dtype=np.float64)
    if X.ndim == 1:
        X = X[:, None]
    vtotal, ctotal = homo - vmin + 1, cmax - homo
    out = np.zeros(3 * X.shape[1])
    _transition_dipoles_block(ao_dipoles, mos, vmin, vtotal, homo + 1, ctotal, X, Y, -np.sqrt(2.0), out, False)
    return out.reshape(X.shape[1], 3)


def transition_dipoles_uks(ao_dipoles, mos_alpha, mos_beta, homo_alpha, homo_beta, vmin, cmax, X, Y=None):
    """Transition dipoles (nstates x 3) of combined UKS excitons (orbitals.cc:804-877): the
    alpha block of each state with the alpha orbitals plus the beta block with the beta
    orbitals, times -1 (no sqrt(2): both spin sectors are explicit)."""
    X = np.asarray(X, dtype=np.float64)
    if X.ndim == 1:
        X = X[:, None]
    va, ca = homo_alpha - vmin + 1, cmax - homo_alpha
    vb, cb = homo_beta - vmin + 1, cmax - homo_beta
    if X.shape[0] != va * ca + vb * cb:
        raise ValueError("transition_dipoles_uks: exciton vector size does not match alpha+beta sector sizes")
    na = va * ca
    Ya = Yb = None
    if Y is not None:
        Y = np.asarray(Y, dtype=np.float64).reshape(X.shape)
        Ya, Yb = Y[:na], Y[na:]
    out = np.zeros(3 * X.shape[1])
    first = True
    for mos, v, c, homo, xs, ys in ((mos_alpha, va, ca, homo_alpha, X[:na], Ya),
                                    (mos_beta, vb, cb, homo_beta, X[na:], Yb)):
        if v * c == 0:
            continue
        _transition_dipoles_block(ao_dipoles, mos, vmin, v, homo + 1, c, xs, ys, -1.0, out, not first)
        first = False
    return out.reshape(X.shape[1], 3)


def oscillator_strengths(omega, dipoles):
    """f = 2/3 Omega |d|^2 per state (Orbitals::Oscillatorstrengths, orbitals.cc:661-673),
    Omega in Hartree and d in e bohr."""
    d = np.asarray(dipoles, dtype=np.float64)
    n = min(len(d), len(omega))
    return np.sum(d[:n] ** 2, axis=1) * 2.0 / 3.0 * np.asarray(omega, dtype=np.float64)[:n]

