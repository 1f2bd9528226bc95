"""CPU restatement of the unrestricted (UKS) BSE operator (TEST INFRASTRUCTURE ONLY).

Only tests/ may use this module, as the reference of the GPU UKS operator.  It restates
BSE_OPERATOR_UKS<cqp, cx, cd, cd2> of xtp/src/libxtp/gwbse/bse_operator_uks.cc block by
block, with the same loops over output pairs and the same Mmn slices and rows:

  setup_block / configure       bse_operator_uks.cc:25-43
  Hqp_row / add_qp_block         :46-71
  add_exchange_block             :73-99   (same spin only)
  add_direct_block               :101-137
  add_direct2_block              :139-177
  add_direct_cross_tda_block     :179-218 (alpha <- beta screened transition densities)
  matmul                         :220-270
  dense_matrix                   :272-281
  diagonal                       :283-352

Index conventions follow the reference: slice m of Mmn is column-major [nn x naux]
(M(m, n, P) = mmn[m, P, n] here), m and n counted from rpamin; a spin block's pair
index is v * ctotal + c; the alpha block comes first.  The same-spin blocks equal the
restricted BSE_OPERATOR of each channel (checked in tests/test_uks_oracle.py against the
restricted oracle, which reproduces the reference's golden operator matrices); the cross-spin
blocks have no golden data (the reference has no UKS operator test) and rest on this
loop-level restatement alone.
"""
from __future__ import annotations

import numpy as np

# BSE_OPERATOR_UKS coefficient sets, bse_operator_uks.h:111-124
UKS_OPERATORS = {
    "tda": (1, 1, 1, 0),     # ExcitonUKSOperator_TDA: Hqp + Hx - Hd (+ cross-spin)
    "btda_b": (0, 1, 0, 1),  # ExcitonUKSOperator_BTDA_B: Hx - Hd2 (+ cross-spin Hd2)
    "hd": (0, 0, 1, 0),      # HdUKSOperator
    "hd2": (0, 0, 0, 1),     # Hd2UKSOperator
    "qp": (1, 0, 0, 0),      # QpUKSOperator
    "hx": (0, 1, 0, 0),      # HxUKSOperator
}


class _Block:
    """SpinBlockInfo of one spin channel (setup_block, bse_operator_uks.cc:25-35)."""

    def __init__(self, homo, vmin, rpamin, cmax, offset):
        self.homo = homo
        self.vmin_rpa = vmin - rpamin
        self.cmin_rpa = homo + 1 - rpamin
        self.vtotal = homo - vmin + 1
        self.ctotal = cmax - (homo + 1) + 1
        self.size = self.vtotal * self.ctotal
        self.offset = offset


def _rows(mmn, m, r0, n):
    """Mmn[m].middleRows(r0, n): an (n x naux) matrix."""
    return mmn[m, :, r0:r0 + n].T


class UKSProblem:
    """Inputs of BSE_OPERATOR_UKS(epsilon_0_inv, Mmn{alpha, beta}, Hqp_alpha, Hqp_beta)
    configured with BSEOperatorUKS_Options{homo_alpha, homo_beta, rpamin, qpmin, vmin, cmax}."""

    def __init__(self, mmn_alpha, mmn_beta, w, hqp_alpha, hqp_beta, homo_alpha, homo_beta,
                 rpamin, vmin, cmax):
        self.ma = np.ascontiguousarray(mmn_alpha, dtype=np.float64)
        self.mb = np.ascontiguousarray(mmn_beta, dtype=np.float64)
        self.w = np.ascontiguousarray(w, dtype=np.float64)
        self.ha = np.asarray(hqp_alpha, dtype=np.float64)
        self.hb = np.asarray(hqp_beta, dtype=np.float64)
        self.alpha = _Block(homo_alpha, vmin, rpamin, cmax, 0)
        self.beta = _Block(homo_beta, vmin, rpamin, cmax, self.alpha.size)
        self.size = self.alpha.size + self.beta.size

    # ---- blocks --------------------------------------------------------------------
    @staticmethod
    def _hqp_row(H, blk, v1, c1):
        r = np.zeros((blk.ctotal, blk.vtotal))
        cq = blk.vtotal
        r[:, v1] += H[cq:cq + blk.ctotal, c1 + cq]
        r[c1, :] -= H[:blk.vtotal, v1]
        return r.reshape(-1, order="F")

    def _qp(self, y, x, blk, H, cqp):
        if cqp == 0:
            return
        for c1 in range(blk.ctotal):
            for v1 in range(blk.vtotal):
                y[v1 * blk.ctotal + c1] += self._hqp_row(H, blk, v1, c1) @ x

    def _exchange(self, y, x, ob, ib, Mo, Mi, pref, cx):
        if cx == 0 or pref == 0.0:
            return
        for v1 in range(ob.vtotal):
            left = pref * _rows(Mo, v1 + ob.vmin_rpa, ob.cmin_rpa, ob.ctotal)
            for v2 in range(ib.vtotal):
                right = _rows(Mi, v2 + ib.vmin_rpa, ib.cmin_rpa, ib.ctotal)
                blk = left @ right.T
                y[v1 * ob.ctotal:(v1 + 1) * ob.ctotal] += blk @ x[v2 * ib.ctotal:(v2 + 1) * ib.ctotal]

    def _direct(self, y, x, ob, ib, Mo, Mi, pref, cd):
        if cd == 0 or pref == 0.0:
            return
        for v1 in range(ob.vtotal):
            for c1 in range(ob.ctotal):
                left = pref * _rows(Mo, c1 + ob.cmin_rpa, ib.cmin_rpa, ib.ctotal)
                right = _rows(Mi, v1 + ob.vmin_rpa, ib.vmin_rpa, ib.vtotal)
                blk = (left * self.w) @ right.T            # (ct_in x vt_in)
                row = blk.reshape(-1, order="F")           # index v2 * ct_in + c2
                y[v1 * ob.ctotal + c1] += row @ x

    def _direct2(self, y, x, ob, ib, Mo, Mi, pref, cd2):
        if cd2 == 0 or pref == 0.0:
            return
        for c1 in range(ob.ctotal):
            left = pref * _rows(Mo, c1 + ob.cmin_rpa, ib.vmin_rpa, ib.vtotal)
            for v1 in range(ob.vtotal):
                right = _rows(Mi, v1 + ob.vmin_rpa, ib.cmin_rpa, ib.ctotal)
                blk = (left * self.w) @ right.T            # (vt_in x ct_in)
                row = blk.reshape(-1, order="C")           # index v2 * ct_in + c2
                y[v1 * ob.ctotal + c1] += row @ x

    def _direct_cross_tda(self, y, x, ob, ib, Mo, Mi, pref, cd):
        if cd == 0 or pref == 0.0:
            return
        for v1 in range(ob.vtotal):
            for c1 in range(ob.ctotal):
                tout = pref * Mo[c1 + ob.cmin_rpa, :, v1 + ob.vmin_rpa]
                acc = 0.0
                for v2 in range(ib.vtotal):
                    tin = _rows(Mi, v2 + ib.vmin_rpa, ib.cmin_rpa, ib.ctotal)
                    acc = acc + (tin @ (self.w * tout)) @ x[v2 * ib.ctotal:(v2 + 1) * ib.ctotal]
                y[v1 * ob.ctotal + c1] += acc

    # ---- operator ------------------------------------------------------------------
    def matmul(self, X, op="tda"):
        cqp, cx, cd, cd2 = UKS_OPERATORS[op] if isinstance(op, str) else op
        if cd != 0 and cd2 != 0:
            raise ValueError("Hamiltonian cannot contain Hd and Hd2 at the same time")
        X = np.asarray(X, dtype=np.float64)
        squeeze = X.ndim == 1
        if squeeze:
            X = X[:, None]
        a, b = self.alpha, self.beta
        xa, xb = X[:a.size], X[a.size:]
        ya = np.zeros_like(xa)
        yb = np.zeros_like(xb)
        self._qp(ya, xa, a, self.ha, cqp)
        self._exchange(ya, xa, a, a, self.ma, self.ma, float(cx), cx)
        self._direct(ya, xa, a, a, self.ma, self.ma, -float(cd), cd)
        self._direct2(ya, xa, a, a, self.ma, self.ma, -float(cd2), cd2)
        self._qp(yb, xb, b, self.hb, cqp)
        self._exchange(yb, xb, b, b, self.mb, self.mb, float(cx), cx)
        self._direct(yb, xb, b, b, self.mb, self.mb, -float(cd), cd)
        self._direct2(yb, xb, b, b, self.mb, self.mb, -float(cd2), cd2)
        self._direct_cross_tda(ya, xb, a, b, self.ma, self.mb, -float(cd), cd)
        self._direct_cross_tda(yb, xa, b, a, self.mb, self.ma, -float(cd), cd)
        self._direct2(ya, xb, a, b, self.ma, self.mb, -float(cd2), cd2)
        self._direct2(yb, xa, b, a, self.mb, self.ma, -float(cd2), cd2)
        Y = np.vstack([ya, yb])
        return Y[:, 0] if squeeze else Y

    def dense(self, op="tda"):
        return self.matmul(np.eye(self.size), op)

    def diagonal(self, op="tda"):
        cqp, cx, cd, cd2 = UKS_OPERATORS[op] if isinstance(op, str) else op
        out = np.zeros(self.size)
        for blk, M, H in ((self.alpha, self.ma, self.ha), (self.beta, self.mb, self.hb)):
            for v in range(blk.vtotal):
                for c in range(blk.ctotal):
                    e = 0.0
                    if cx != 0:
                        r = M[v + blk.vmin_rpa, :, blk.cmin_rpa + c]
                        e += cx * float(r @ r)
                    if cqp != 0:
                        cq = blk.vtotal
                        e += H[c + cq, c + cq] - H[v, v]
                    if cd != 0:
                        e -= float((M[c + blk.cmin_rpa, :, blk.cmin_rpa + c] * self.w)
                                   @ M[v + blk.vmin_rpa, :, blk.vmin_rpa + v])
                    if cd2 != 0:
                        e -= float((M[c + blk.cmin_rpa, :, blk.vmin_rpa + v] * self.w)
                                   @ M[v + blk.vmin_rpa, :, blk.cmin_rpa + c])
                    out[blk.offset + v * blk.ctotal + c] = e
        return out


def full_bse_dense_roots(A, B, nmax):
    """The dense fallback of BSE_UKS::Solve_excitons_uks_BTDA (bse_uks.cc:313-406):
    eigenpairs of [[A, B], [-B, -A]] with a positive real part and |imag| < 1e-8, the
    lowest nmax, phase fixed so that the largest |X_k| is positive, normalised to
    |X|^2 - |Y|^2 = 1."""
    n = A.shape[0]
    H = np.block([[A, B], [-B, -A]])
    ev, vec = np.linalg.eig(H)
    roots = sorted((ev[i].real, i) for i in range(2 * n) if abs(ev[i].imag) < 1e-8 and ev[i].real > 0.0)
    if not roots:
        raise RuntimeError("Dense full UKS-BSE diagonalization produced no positive real roots.")
    roots = roots[:min(nmax, len(roots))]
    lam = np.array([r[0] for r in roots])
    Xs, Ys = [], []
    for _, col in roots:
        v = vec[:, col].real
        X, Y = v[:n].copy(), v[n:].copy()
        if X[np.argmax(np.abs(X))] < 0.0:
            X, Y = -X, -Y
        nrm = X @ X - Y @ Y
        if abs(nrm) < 1e-12:
            raise RuntimeError("Dense full UKS-BSE eigenvector has near-zero (X^2-Y^2) norm.")
        s = 1.0 / np.sqrt(abs(nrm))
        Xs.append(X * s)
        Ys.append(Y * s)
    return lam, np.array(Xs).T, np.array(Ys).T
