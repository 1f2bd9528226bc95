"""Adjoint (Hellmann-Feynman) eigenvalue gradients on the GPU, behind torch.autograd,
against central finite differences (step 1e-5) and an FP64 CPU reference gradient."""
import numpy as np
import pytest

import oracle
from votca_gb300.synthetic import Problem, dense_screening

pytestmark = pytest.mark.gpu

V, C, NAUX, NMO, NROOTS = 4, 10, 20, 14, 3
COEF = (1, 2, 1, 0)


def setup(seed=31, dense=False):
    import torch

    from votca_gb300.bse_operator import BSEOperator_Options

    p = Problem(v=V, c=C, naux=NAUX, nmo=NMO, seed=seed)
    opt = BSEOperator_Options(homo=V - 1, rpamin=0, qpmin=0, vmin=0, cmax=V + C - 1)
    mmn = torch.tensor(p.mmn, requires_grad=True)
    hqp = torch.tensor(p.hqp[:V + C, :V + C].copy(), requires_grad=True)
    if dense:
        eps, Q, lam = dense_screening(seed, NAUX)
        w = torch.tensor(np.eye(NAUX) - np.linalg.inv(eps), requires_grad=True)
    else:
        w = torch.tensor(p.w.copy(), requires_grad=True)
    return p, opt, mmn, hqp, w


def dense_eigs(mmn, hqp, w):
    """Lowest eigenvalues from the oracle-assembled operator (FP64 CPU).  A dense W
    is folded exactly into the vv block (M(v1, v, .) <- W M(v1, v, .)), which is
    the operator the dense-screening handle applies.  A single perturbed Mmn entry
    makes the operator non-symmetric; its symmetric part has the same first-order
    eigenvalue change (x^T E x = x^T E^T x), so the symmetrised matrix is used."""
    if w.ndim == 2:
        mmn = mmn.copy()
        mmn[:V, :, :V] = np.einsum("pq,mqn->mpn", w, mmn[:V, :, :V])
        w = np.ones(w.shape[0])
    prob = oracle.BSEProblem(mmn, w, hqp, V, C)
    H = prob.dense("singlet")
    return np.linalg.eigvalsh(0.5 * (H + H.T))[:NROOTS]


def fd_tolerance(fd, g, lam, h):
    """1e-6 relative, plus the rounding floor of a central difference of FP64
    eigenvalues: 16 eps sum_k |g_k Omega_k| / (2 h)."""
    return 1e-6 * abs(fd) + 16 * np.finfo(float).eps * float(np.sum(np.abs(g * lam))) / (2 * h)


def cpu_reference_gradient(mmn, hqp, w, g):
    """x^T (dA) x by brute force on the dense operator: dOmega/dtheta for each
    stored Mmn entry via the analytic bilinear forms (FP64, numpy)."""
    prob = oracle.BSEProblem(mmn, w, hqp, V, C)
    ev, U = np.linalg.eigh(prob.dense("singlet"))
    X = U[:, :NROOTS]
    gm = np.zeros_like(mmn)
    gw = np.zeros_like(w)
    for k in range(NROOTS):
        x = X[:, k].reshape(V, C)
        Mvc = mmn[:V, :, V:V + C]                  # (v, P, c)
        Mvv = mmn[:V, :, :V]                       # (v, P, v')
        Mcc = mmn[V:V + C, :, V:V + C]             # (c, P, c')
        z = np.einsum("vpc,vc->p", Mvc, x)
        gm[:V, :, V:V + C] += g[k] * 2 * COEF[1] * np.einsum("p,vc->vpc", z, x)
        S = np.einsum("cpd,ed->pec", Mcc, x)      # S[P][v'][c] = sum_c' M(c,c',P) x[v'][c']
        Q = np.einsum("vc,pec->pve", x, S)         # Q[P][v][v']
        gm[:V, :, :V] += g[k] * (-COEF[2]) * np.einsum("p,pve->vpe", w, Q)
        gw += g[k] * (-COEF[2]) * np.einsum("pve,vpe->p", Q, Mvv)
        T = np.einsum("vpe,ed->pvd", Mvv, x) * w[:, None, None]   # (G^P X)[v][c']
        gm[V:V + C, :, V:V + C] += g[k] * (-COEF[2]) * np.einsum("vc,pvd->cpd", x, T)
    return gm, gw


def test_adjoint_matches_cpu_reference_and_finite_differences():
    import torch

    from votca_gb300.adjoint import bse_eigenvalues

    p, opt, mmn, hqp, w = setup()
    lam = bse_eigenvalues(mmn, hqp, w, opt, NROOTS, COEF, 1e-10)
    ref = dense_eigs(p.mmn, p.hqp[:V + C, :V + C], p.w)
    assert np.max(np.abs(lam.detach().numpy() - ref)) < 1e-11
    g = np.array([0.7, -1.3, 2.1])
    (lam * torch.tensor(g)).sum().backward()
    gm, gh, gw = mmn.grad.numpy(), hqp.grad.numpy(), w.grad.numpy()
    # FP64 CPU reference gradient (full tensors)
    gm_ref, gw_ref = cpu_reference_gradient(p.mmn, p.hqp[:V + C, :V + C].copy(), p.w, g)
    assert np.allclose(gm, gm_ref, rtol=1e-9, atol=1e-12)
    assert np.allclose(gw, gw_ref, rtol=1e-9, atol=1e-12)
    # central finite differences, step 1e-5, on 64 random Mmn entries in the BSE window
    rng = np.random.default_rng(0)
    f = lambda mm, hh, ww: float(g @ dense_eigs(mm, hh, ww))
    h = 1e-5
    idx = [(rng.integers(0, V + C), rng.integers(0, NAUX), rng.integers(0, V + C)) for _ in range(64)]
    for (m, P, n) in idx:
        mp, mm_ = p.mmn.copy(), p.mmn.copy()
        mp[m, P, n] += h
        mm_[m, P, n] -= h
        fd = (f(mp, p.hqp[:V + C, :V + C], p.w) - f(mm_, p.hqp[:V + C, :V + C], p.w)) / (2 * h)
        assert abs(fd - gm[m, P, n]) <= fd_tolerance(fd, g, ref, h), (m, P, n, fd, gm[m, P, n])
    # QP energies (diagonal of Hqp) and screening weights
    for i in range(V + C):
        hp, hm = p.hqp[:V + C, :V + C].copy(), p.hqp[:V + C, :V + C].copy()
        hp[i, i] += h
        hm[i, i] -= h
        fd = (f(p.mmn, hp, p.w) - f(p.mmn, hm, p.w)) / (2 * h)
        assert abs(fd - gh[i, i]) <= fd_tolerance(fd, g, ref, h)
    for P in rng.integers(0, NAUX, 8):
        wp, wm = p.w.copy(), p.w.copy()
        wp[P] += h
        wm[P] -= h
        fd = (f(p.mmn, p.hqp[:V + C, :V + C], wp) - f(p.mmn, p.hqp[:V + C, :V + C], wm)) / (2 * h)
        assert abs(fd - gw[P]) <= fd_tolerance(fd, g, ref, h)


def test_adjoint_dense_screening_finite_differences():
    import torch

    from votca_gb300.adjoint import bse_eigenvalues

    p, opt, mmn, hqp, W = setup(seed=17, dense=True)
    lam = bse_eigenvalues(mmn, hqp, W, opt, NROOTS, COEF, 1e-10)
    g = np.array([1.0, 0.5, -0.25])
    (lam * torch.tensor(g)).sum().backward()
    gW = W.grad.numpy()
    Wn = W.detach().numpy()
    lam0 = dense_eigs(p.mmn, p.hqp[:V + C, :V + C], Wn)
    assert np.max(np.abs(lam.detach().numpy() - lam0)) < 1e-11
    f = lambda ww: float(g @ dense_eigs(p.mmn, p.hqp[:V + C, :V + C], ww))
    h = 1e-5
    rng = np.random.default_rng(1)
    for _ in range(16):
        P, Q = rng.integers(0, NAUX, 2)
        wp, wm = Wn.copy(), Wn.copy()
        # W is symmetric: perturb the pair, the gradient of the pair is gW[P,Q] + gW[Q,P]
        wp[P, Q] += h
        wm[P, Q] -= h
        if P != Q:
            wp[Q, P] += h
            wm[Q, P] -= h
        fd = (f(wp) - f(wm)) / (2 * h)
        an = gW[P, Q] + (gW[Q, P] if P != Q else 0.0)
        assert abs(fd - an) <= fd_tolerance(fd, g, lam0, h), (P, Q, fd, an)
