"""Adjoint gradients at the medium workload (v=64, c=512, Naux=2048, Nmo=576):
the lowest 5 TDA singlet energies differentiated with respect to Mmn (vc, vv
and cc blocks), the QP energies and the screening weights.

The GPU gradient (torch.autograd backward -> bse_op_eig_gradient) is checked
(1) against an FP64 CPU evaluation of x_k^T (dH/dtheta) x_k for each sampled
entry, written out entry by entry from the operator's bilinear forms, and
(2) against central finite differences (step 1e-5) of FP64 GPU solves on 64
sampled entries.  An off-diagonal vv/cc entry is perturbed together with its
(m, n) mirror so that the perturbed operator stays symmetric; the difference
is then compared with the sum of the two gradient entries.
"""
import time

import numpy as np
import pytest

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

V, C, NAUX, NMO, NROOTS = 64, 512, 2048, 576, 5
COEF = (1, 2, 1, 0)
H = 1e-5


def _ctx(mmn, w, hqp, opt):
    from votca_gb300 import bse_operator as bo

    return bo.GpuBSEContext(w, bo.TCMatrix_gwbse(mmn), hqp, opt, precision=bo.PRECISION_FP64)


def _energy(mmn, w, hqp, opt, guess, g):
    from votca_gb300 import bse_operator as bo
    from votca_gb300.davidson import DavidsonSolver

    ctx = _ctx(mmn, w, hqp, opt)
    ds = DavidsonSolver()
    ds.set_tolerance(1e-9)
    ds.set_max_search_space(10 * NROOTS)
    lam, _ = ds.solve(bo.SingletOperator_TDA(ctx), NROOTS, initial_guess=guess)
    ctx.close()
    assert ds.info() == "Success"
    return float(g @ lam)


def test_adjoint_c1_fd_and_cpu_reference():
    import torch

    from votca_gb300 import bse_operator as bo
    from votca_gb300.adjoint import BSEEigenvalues
    from votca_gb300.davidson import DavidsonSolver
    from votca_gb300.synthetic import mmn_tensor_torch, qp_energies, screening_w

    t_start = time.perf_counter()
    seed = 5
    mmn = mmn_tensor_torch(seed, NAUX, NMO)
    w = screening_w(seed, NAUX)
    hqp = np.diag(qp_energies(seed, V, C))
    opt = bo.BSEOperator_Options(homo=V - 1, rpamin=0, qpmin=0, vmin=0, cmax=V + C - 1)
    g = np.array([1.0, -0.6, 0.8, 1.3, -0.4])

    tm = torch.from_numpy(mmn).requires_grad_(True)
    th = torch.from_numpy(hqp.copy()).requires_grad_(True)
    tw = torch.from_numpy(w.copy()).requires_grad_(True)
    lam = BSEEigenvalues.apply(tm, th, tw, opt, NROOTS, COEF, 1e-10, 0)
    (lam * torch.tensor(g)).sum().backward()
    gm, gh, gw = tm.grad.numpy(), th.grad.numpy(), tw.grad.numpy()
    lam = lam.detach().numpy()

    # eigenvectors of the same solve for the CPU reference and the warm starts
    ctx = _ctx(mmn, w, hqp, opt)
    ds = DavidsonSolver()
    ds.set_tolerance(1e-10)
    ds.set_max_search_space(10 * NROOTS)
    lam2, X = ds.solve(bo.SingletOperator_TDA(ctx), NROOTS)
    ctx.close()
    np.testing.assert_allclose(lam2, lam, rtol=0, atol=1e-12)
    xs = [X[:, k].reshape(V, C) for k in range(NROOTS)]

    rng = np.random.default_rng(11)
    Mvc = mmn[:V, :, V:]  # (v, P, c) views
    z = [np.einsum("vpc,vc->p", Mvc, x) for x in xs]

    def ref_vc(v, P, c):
        return sum(g[k] * 2 * COEF[1] * z[k][P] * xs[k][v, c] for k in range(NROOTS))

    def ref_vv(v1, P, v2):  # -cd w_P x[v1,:] M(c, c', P) x[v2,:]
        Mc = mmn[V:, P, V:]
        return sum(g[k] * (-COEF[2]) * w[P] * (xs[k][v1] @ Mc @ xs[k][v2]) for k in range(NROOTS))

    def ref_cc(c1, P, c2):  # -cd w_P x[:,c1] M(v, v', P) x[:,c2]
        Mv = mmn[:V, P, :V]
        return sum(g[k] * (-COEF[2]) * w[P] * (xs[k][:, c1] @ Mv @ xs[k][:, c2]) for k in range(NROOTS))

    def ref_w(P):
        Mc, Mv = mmn[V:, P, V:], mmn[:V, P, :V]
        return sum(g[k] * (-COEF[2]) * np.sum((xs[k] @ Mc @ xs[k].T) * Mv) for k in range(NROOTS))

    def ref_qp(i):
        if i < V:
            return sum(-g[k] * np.sum(xs[k][i] ** 2) for k in range(NROOTS))
        return sum(g[k] * np.sum(xs[k][:, i - V] ** 2) for k in range(NROOTS))

    # 64 sampled entries: 16 vc, 16 vv, 16 cc, 8 QP energies, 8 screening weights.
    # The low excitons sit on few (v, c) pairs, so the orbital indices are drawn
    # from the pairs that carry the largest amplitudes (a random pair has a
    # gradient near zero, which a difference cannot resolve); P is uniform.
    amp = sum(np.abs(x) for x in xs)
    top = np.argsort(amp.ravel())[::-1][:24]
    top_v, top_c = top // C, top % C
    pick = lambda a: int(a[rng.integers(len(a))])
    entries = []
    for _ in range(16):
        t = pick(top)
        entries.append(("vc", int(t // C), int(rng.integers(NAUX)), V + int(t % C)))
    for _ in range(16):
        entries.append(("vv", pick(top_v), int(rng.integers(NAUX)), pick(top_v)))
    for _ in range(16):
        entries.append(("cc", V + pick(top_c), int(rng.integers(NAUX)), V + pick(top_c)))
    for i in [pick(top_v) for _ in range(4)] + [V + pick(top_c) for _ in range(4)]:
        entries.append(("qp", int(i), 0, int(i)))
    for P in rng.integers(0, NAUX, 8):
        entries.append(("w", 0, int(P), 0))

    # (1) CPU reference, entry by entry
    for kind, m, P, n in entries:
        if kind == "vc":
            an, ref = gm[m, P, n], ref_vc(m, P, n - V)
        elif kind == "vv":
            an, ref = gm[m, P, n], ref_vv(m, P, n)
        elif kind == "cc":
            an, ref = gm[m, P, n], ref_cc(m - V, P, n - V)
        elif kind == "qp":
            an, ref = gh[m, m], ref_qp(m)
        else:
            an, ref = gw[P], ref_w(P)
        assert abs(an - ref) <= 1e-9 * abs(ref) + 1e-13, (kind, m, P, n, an, ref)

    # (2) central finite differences of FP64 solves, warm-started from X
    eps = np.finfo(float).eps
    # rounding floor of a central difference of FP64 eigenvalues
    floor = 64 * eps * float(np.sum(np.abs(g * lam))) / (2 * H)
    worst = 0.0
    errs, mags = [], []
    for kind, m, P, n in entries:
        vals = []
        for sgn in (1.0, -1.0):
            if kind in ("vc", "vv", "cc"):
                old = (mmn[m, P, n], mmn[n, P, m])
                mmn[m, P, n] += sgn * H
                if kind != "vc" and m != n:
                    mmn[n, P, m] += sgn * H
                vals.append(_energy(mmn, w, hqp, opt, X, g))
                mmn[m, P, n], mmn[n, P, m] = old
            elif kind == "qp":
                hp = hqp.copy()
                hp[m, m] += sgn * H
                vals.append(_energy(mmn, w, hp, opt, X, g))
            else:
                wp = w.copy()
                wp[P] += sgn * H
                vals.append(_energy(mmn, wp, hqp, opt, X, g))
        fd = (vals[0] - vals[1]) / (2 * H)
        if kind == "vc" or (kind in ("vv", "cc") and m == n):
            an = gm[m, P, n]
        elif kind in ("vv", "cc"):
            an = gm[m, P, n] + gm[n, P, m]
        elif kind == "qp":
            an = gh[m, m]
        else:
            an = gw[P]
        tol = 1e-6 * abs(fd) + floor
        worst = max(worst, abs(fd - an) / tol)
        errs.append(abs(fd - an) / max(abs(fd), 1e-300))
        mags.append(abs(an))
        assert abs(fd - an) <= tol, (kind, m, P, n, fd, an, tol)
    print(f"\nC1 adjoint: 64 entries, worst |fd - grad| / tol = {worst:.3f}, median relative "
          f"|fd - grad| / |fd| {np.median(errs):.2e}, |grad| range {min(mags):.2e}..{max(mags):.2e}, "
          f"floor {floor:.2e}, {time.perf_counter() - t_start:.1f} s")
