"""Unrestricted (UKS) BSE operator on the GPU, mirroring VOTCA-XTP's BSE_OPERATOR_UKS
(xtp/include/votca/xtp/bse_operator_uks.h, xtp/src/libxtp/gwbse/bse_operator_uks.cc) and
the solve drivers of BSE_UKS (xtp/src/libxtp/gwbse/bse_uks.cc).

  BSEOperatorUKS_Options     bse_operator_uks.h:31-38
  TCMatrix_gwbse_spin        threecenter.h:144-155 (alpha and beta Mmn)
  GpuBSEContextUKS           the staged operator (bse_uks_op_create); several coefficient
                             sets share one context, as BSE_OPERATOR_UKS instances share the
                             caller's epsilon_0_inv, Mmn and Hqp references
  BSE_OPERATOR_UKS + presets ExcitonUKSOperator_TDA <1,1,1,0>, ExcitonUKSOperator_BTDA_B
                             <0,1,0,1>, HdUKSOperator, Hd2UKSOperator, QpUKSOperator,
                             HxUKSOperator (bse_operator_uks.h:111-124)
  solve_excitons_uks_tda     BSE_UKS::Solve_excitons_uks_TDA, bse_uks.cc:218-231
  solve_excitons_uks_btda    BSE_UKS::Solve_excitons_uks_BTDA, bse_uks.cc:291-440 (dense
                             solve up to dim 128, else the HAM Davidson with the ranked guess)
  exciton_weights_uks        the composition BSE_UKS::Analyze_excitons_uks reports per root
                             (PrintWeightsUKS, bse_uks.cc:520-595, 597-638): sector weights and
                             the largest transitions, as data instead of log lines

Vectors are [x_alpha; x_beta]: alpha pairs first, pair index v * ctotal + c per channel.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from .bse import DavidsonOptions, _solver, full_bse_ranked_guess
from .bse_operator import BSE_OPERATOR, PRECISION_FP64, TCMatrix_gwbse, HamiltonianOperator, _p


@dataclass
class BSEOperatorUKS_Options:
    homo_alpha: int
    homo_beta: int
    rpamin: int
    qpmin: int
    vmin: int
    cmax: int


class TCMatrix_gwbse_spin:
    """Alpha and beta Mmn of one auxiliary basis."""

    def __init__(self, alpha: TCMatrix_gwbse, beta: TCMatrix_gwbse):
        self.alpha, self.beta = alpha, beta


def _mmn_args(Mmn: TCMatrix_gwbse):
    desc = _lib.bse_mmn_desc(Mmn.auxsize(), Mmn.get_mmin(), Mmn.get_mmax(), Mmn.get_nmin(), Mmn.get_nmax())
    ptrs = (_lib.c_dp * Mmn.msize())(*[
        ctypes.cast(Mmn.data.ctypes.data + m * Mmn.data.strides[0], _lib.c_dp) for m in range(Mmn.msize())])
    return desc, ptrs


class GpuBSEContextUKS:
    """Device-resident staging of (epsilon_0_inv, Mmn alpha/beta, Hqp alpha/beta) for the
    unrestricted BSE window given by BSEOperatorUKS_Options."""

    def __init__(self, epsilon_0_inv, Mmn: TCMatrix_gwbse_spin, Hqp_alpha, Hqp_beta, opt: BSEOperatorUKS_Options,
                 precision=PRECISION_FP64, dense_screening=None):
        L = _lib.load()
        self._L = L
        da, pa = _mmn_args(Mmn.alpha)
        db, pb = _mmn_args(Mmn.beta)
        ha = np.asfortranarray(Hqp_alpha, dtype=np.float64)
        hb = np.asfortranarray(Hqp_beta, dtype=np.float64)
        o = _lib.bse_uks_options(opt.homo_alpha, opt.homo_beta, opt.rpamin, opt.qpmin, opt.vmin, opt.cmax)
        h = ctypes.c_void_p()
        if dense_screening is not None:
            w = np.asfortranarray(dense_screening, dtype=np.float64)
            create = L.bse_uks_op_create_dense_screening
        else:
            if epsilon_0_inv is None:
                raise _lib.BSEError(1, "GpuBSEContextUKS: epsilon_0_inv or dense_screening is required")
            w = np.ascontiguousarray(epsilon_0_inv, dtype=np.float64)
            create = L.bse_uks_op_create
        _lib.check(create(ctypes.byref(da), pa, ctypes.byref(db), pb, _p(w), _p(ha), ha.shape[0], ha.shape[0],
                          _p(hb), hb.shape[0], hb.shape[0], ctypes.byref(o), precision, ctypes.byref(h)))
        self.handle = h
        n = ctypes.c_int64()
        _lib.check(L.bse_op_size(h, ctypes.byref(n)))
        self.size = n.value
        self.size_alpha = (opt.homo_alpha - opt.vmin + 1) * (opt.cmax - opt.homo_alpha)
        self.size_beta = self.size - self.size_alpha
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


class BSE_OPERATOR_UKS(BSE_OPERATOR):
    """BSE_OPERATOR_UKS<cqp, cx, cd, cd2> on a GpuBSEContextUKS: same-spin
    cqp Hqp + cx Hx - cd Hd - cd2 Hd2 per channel plus the cross-spin terms."""

    def dense_matrix(self):
        """BSE_OPERATOR_UKS::dense_matrix (bse_operator_uks.cc:272-281): the product with
        every unit vector."""
        return self.matmul(np.eye(self.rows(), order="F"))


def _preset(name, c):
    return type(name, (BSE_OPERATOR_UKS,), {"cqp": c[0], "cx": c[1], "cd": c[2], "cd2": c[3]})


ExcitonUKSOperator_TDA = _preset("ExcitonUKSOperator_TDA", (1, 1, 1, 0))
ExcitonUKSOperator_BTDA_B = _preset("ExcitonUKSOperator_BTDA_B", (0, 1, 0, 1))
HdUKSOperator = _preset("HdUKSOperator", (0, 0, 1, 0))
Hd2UKSOperator = _preset("Hd2UKSOperator", (0, 0, 0, 1))
QpUKSOperator = _preset("QpUKSOperator", (1, 0, 0, 0))
HxUKSOperator = _preset("HxUKSOperator", (0, 1, 0, 0))

# BSE_UKS::Solve_excitons_uks_BTDA solves densely up to this dimension (bse_uks.cc:311-313)
DENSE_THRESHOLD = 128


def solve_excitons_uks_tda(ctx: GpuBSEContextUKS, opt: DavidsonOptions):
    """Lowest opt.nmax roots of the UKS TDA Hamiltonian: (eigenvalues, eigenvectors, solver)."""
    ds = _solver(opt)
    evals, evecs = ds.solve(ExcitonUKSOperator_TDA(ctx), opt.nmax)
    return evals, evecs, ds


def _dense_full_bse(A, B, nmax):
    # dense branch of Solve_excitons_uks_BTDA (bse_uks.cc:313-406): eigenpairs of
    # [[A, B], [-B, -A]] with a positive real part and |imag| < 1e-8, lowest first, phase so
    # that the largest |X_k| is positive, |X|^2 - |Y|^2 = 1
    n = A.shape[0]
    H = np.block([[A, B], [-B, -A]])
    ev, vec = np.linalg.eig(H)
    roots = sorted((ev[i].real, i) for i in range(2 * n) if abs(ev[i].imag) < 1e-8 and ev[i].real > 0.0)
    if not roots:
        raise RuntimeError("Dense full UKS-BSE diagonalization produced no positive real roots.")
    roots = roots[:min(nmax, len(roots))]
    lam = np.empty(len(roots))
    X = np.zeros((n, len(roots)))
    Y = np.zeros((n, len(roots)))
    for j, (val, col) in enumerate(roots):
        v = vec[:, col].real
        x, y = v[:n].copy(), v[n:].copy()
        if x[np.argmax(np.abs(x))] < 0.0:
            x, y = -x, -y
        nrm = x @ x - y @ y
        if abs(nrm) < 1e-12:
            raise RuntimeError("Dense full UKS-BSE eigenvector has near-zero (X^2-Y^2) norm.")
        s = 1.0 / np.sqrt(abs(nrm))
        lam[j], X[:, j], Y[:, j] = val, x * s, y * s
    return lam, X, Y


def solve_excitons_uks_btda(ctx: GpuBSEContextUKS, opt: DavidsonOptions):
    """Lowest opt.nmax full-BSE roots: (eigenvalues, X, Y, solver or None for the dense branch)
    with |X|^2 - |Y|^2 = 1 per root."""
    A, B = ExcitonUKSOperator_TDA(ctx), ExcitonUKSOperator_BTDA_B(ctx)
    if A.rows() <= DENSE_THRESHOLD:
        lam, X, Y = _dense_full_bse(A.dense_matrix(), B.dense_matrix(), opt.nmax)
        return lam, X, Y, None
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


@dataclass
class UKSContribution:
    weight: float
    is_alpha: bool
    v: int  # index in the spin block's occupied range (vmin + v is the level)
    c: int  # index in the spin block's virtual range (homo + 1 + c is the level)
    homo_minus: int  # HOMO-<homo_minus>
    lumo_plus: int   # LUMO+<lumo_plus>


def exciton_weights_uks(opt: BSEOperatorUKS_Options, X, Y=None, min_print_weight=0.5, max_print=8):
    """Per root: (alpha-sector weight, beta-sector weight, the largest contributions).
    weights = |X|^2 (TDA) or |X|^2 - |Y|^2 (full BSE) per pair; contributions with
    |weight| > min_print_weight (the gwbse option print_weight, default 0.5), sorted by |weight|
    and cut at max_print (8 in the reference); the number above the threshold that were cut is
    returned too."""
    X = np.asarray(X, dtype=np.float64)
    if X.ndim == 1:
        X = X[:, None]
    w_all = X * X
    if Y is not None:
        Y = np.asarray(Y, dtype=np.float64).reshape(X.shape)
        w_all = w_all - Y * Y
    blocks = []
    off = 0
    for homo, alpha in ((opt.homo_alpha, True), (opt.homo_beta, False)):
        vt, ct = homo - opt.vmin + 1, opt.cmax - homo
        blocks.append((alpha, homo, vt, ct, off))
        off += vt * ct
    if off != X.shape[0]:
        raise ValueError("exciton_weights_uks: vectors do not match the UKS window")
    out = []
    for k in range(X.shape[1]):
        w = w_all[:, k]
        sectors = []
        contribs = []
        for alpha, homo, vt, ct, o in blocks:
            sectors.append(float(np.sum(w[o:o + vt * ct])))
            for i in range(vt * ct):
                if abs(w[o + i]) > min_print_weight:
                    v, c = i // ct, i % ct
                    contribs.append(UKSContribution(float(w[o + i]), alpha, v, c,
                                                    homo - (opt.vmin + v), c))
        contribs.sort(key=lambda t: abs(t.weight), reverse=True)
        out.append({"alpha_weight": sectors[0], "beta_weight": sectors[1],
                    "contributions": contribs[:max_print],
                    "more_above_threshold": max(0, len(contribs) - max_print)})
    return out
