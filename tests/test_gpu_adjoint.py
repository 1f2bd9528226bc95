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


def _dense_ab(mmn, hqp, w):
    """The singlet A and B blocks from the oracle (symmetric parts, as in dense_eigs)."""
    prob = oracle.BSEProblem(mmn, w, hqp, V, C)
    A, B = prob.dense("singlet"), prob.dense("singlet_b")
    return 0.5 * (A + A.T), 0.5 * (B + B.T)


def full_eigs(mmn, hqp, w):
    """The lowest positive roots of [[A, B], [-B, -A]] through the symmetric form: with
    A - B = L L^T, Omega^2 are the eigenvalues of L^T (A + B) L (similar to (A - B)(A + B));
    a symmetric eigensolver keeps the finite differences at the rounding floor below."""
    A, B = _dense_ab(mmn, hqp, w)
    L = np.linalg.cholesky(A - B)
    return np.sqrt(np.linalg.eigvalsh(L.T @ (A + B) @ L))[:NROOTS]


def cpu_reference_gradient_full(mmn, hqp, w, X, Y, g):
    """dOmega = X^T dA X + Y^T dA Y + X^T (dB + dB^T) Y with torch's CPU autograd in FP64 on the
    operator assembled element by element from Mmn (Hx, Hd, Hd2 as bse_operator.cc defines them).
    A single Mmn entry perturbs B unsymmetrically; the first-order change of an eigenvalue of
    [[A, B], [-B, -A]] (left eigenvector J z) then sees the symmetric part, hence dB + dB^T
    (2 X^T dB Y for a symmetric perturbation)."""
    import torch

    M = torch.tensor(mmn, requires_grad=True)
    W = torch.tensor(w, requires_grad=True)
    H = torch.tensor(hqp)
    Mvc, Mvv = M[:V, :, V:V + C], M[:V, :, :V]
    Mcc, Mcv = M[V:V + C, :, V:V + C], M[V:V + C, :, :V]
    n = V * C
    Hx = torch.einsum("vpc,wpd->vcwd", Mvc, Mvc).reshape(n, n)
    Hd = torch.einsum("p,cpd,vpw->vcwd", W, Mcc, Mvv).reshape(n, n)
    Hd2 = torch.einsum("p,vpd,cpw->vcwd", W, Mvc, Mcv).reshape(n, n)
    Hqp = (torch.einsum("vw,cd->vcwd", torch.eye(V, dtype=H.dtype), H[V:, V:])
           - torch.einsum("vw,cd->vcwd", H[:V, :V], torch.eye(C, dtype=H.dtype))).reshape(n, n)
    A = Hqp + 2 * Hx - Hd
    B = 2 * Hx - Hd2
    Xt, Yt = torch.tensor(X), torch.tensor(Y)
    om = (torch.einsum("ik,ij,jk->k", Xt, A, Xt) + torch.einsum("ik,ij,jk->k", Yt, A, Yt)
          + torch.einsum("ik,ij,jk->k", Xt, B + B.T, Yt))
    (om * torch.tensor(g)).sum().backward()
    return om.detach().numpy(), M.grad.numpy(), W.grad.numpy()


def test_full_bse_adjoint_matches_cpu_reference_and_finite_differences():
    """Full BSE: the gradient of sum g_k Omega_k (bse_op_eig_gradient_full behind
    torch.autograd) against the FP64 CPU autograd reference and central differences of the
    dense [[A, B], [-B, -A]] eigenvalues (step 1e-5)."""
    import torch

    from votca_gb300.adjoint import BSEFullEigenvalues

    p, opt, mmn, hqp, w = setup(seed=43)
    hq = p.hqp[:V + C, :V + C].copy()
    lam = BSEFullEigenvalues.apply(mmn, hqp, w, opt, NROOTS, (1, 2, 1, 0), (0, 2, 0, 1), 1e-10, 0)
    ref = full_eigs(p.mmn, hq, p.w)
    assert np.max(np.abs(lam.detach().numpy() - ref)) < 1e-10
    g = np.array([0.9, -0.4, 1.7])
    (lam * torch.tensor(g)).sum().backward()
    gm, gw = mmn.grad.numpy(), w.grad.numpy()
    # the CPU reference at the eigenvectors of the same solve
    from votca_gb300 import bse_operator as bo
    from votca_gb300.bse import DavidsonOptions, solve_nonhermitian_davidson

    ctx = bo.GpuBSEContext(p.w, bo.TCMatrix_gwbse(p.mmn), hq, opt)
    lam2, X, Y, _ = solve_nonhermitian_davidson(bo.SingletOperator_TDA(ctx), bo.SingletOperator_BTDA_B(ctx),
                                                DavidsonOptions(davidson_tolerance=1e-10, nmax=NROOTS))
    om, gm_ref, gw_ref = cpu_reference_gradient_full(p.mmn, hq, p.w, X, Y, g)
    assert np.allclose(om, lam2, atol=1e-10)
    assert np.allclose(gm, gm_ref, rtol=1e-8, atol=1e-11), np.abs(gm - gm_ref).max()
    assert np.allclose(gw, gw_ref, rtol=1e-8, atol=1e-11), np.abs(gw - gw_ref).max()
    # the cv block (read only by the Hd2 term of B) carries gradient
    assert np.abs(gm[V:V + C, :, :V]).max() > 0
    f = lambda mm, ww: float(g @ full_eigs(mm, hq, ww))
    h = 1e-5
    rng = np.random.default_rng(2)
    idx = [(rng.integers(0, V + C), rng.integers(0, NAUX), rng.integers(0, V + C)) for _ in range(48)]
    for (m, P, n) in idx:
        mp, mm_ = p.mmn.copy(), p.mmn.copy()
        mp[m, P, n] += h
        mm_[m, P, n] -= h
        fd = (f(mp, p.w) - f(mm_, p.w)) / (2 * h)
        assert abs(fd - gm[m, P, n]) <= fd_tolerance(fd, g, ref, h), (m, P, n, fd, gm[m, P, n])
    for P in rng.integers(0, NAUX, 8):
        wp, wm = p.w.copy(), p.w.copy()
        wp[P] += h
        wm[P] -= h
        fd = (f(p.mmn, wp) - f(p.mmn, wm)) / (2 * h)
        assert abs(fd - gw[P]) <= fd_tolerance(fd, g, ref, h), (P, fd, gw[P])


def test_device_gradient_blocks_match_host_gradient():
    """bse_op_eig_gradient_device (block layouts on the device) against the Mmn-shaped host
    gradient, for the TDA and the full-BSE forms."""
    import ctypes

    import torch

    from votca_gb300 import _lib
    from votca_gb300 import bse_operator as bo
    from votca_gb300.bse import DavidsonOptions, solve_nonhermitian_davidson

    p, opt, _, _, _ = setup(seed=47)
    hq = p.hqp[:V + C, :V + C].copy()
    ctx = bo.GpuBSEContext(p.w, bo.TCMatrix_gwbse(p.mmn), hq, opt)
    L = ctx._L
    lam, X, Y, _ = solve_nonhermitian_davidson(bo.SingletOperator_TDA(ctx), bo.SingletOperator_BTDA_B(ctx),
                                               DavidsonOptions(davidson_tolerance=1e-10, nmax=NROOTS))
    g = np.array([1.0, 2.0, -0.5])
    a = (ctypes.c_int32 * 4)(1, 2, 1, 0)
    b = (ctypes.c_int32 * 4)(0, 2, 0, 1)
    n = V * C
    for full in (False, True):
        gm = np.zeros(p.mmn.shape)
        gh = np.zeros((V + C, V + C), order="F")
        gw = np.zeros(NAUX)
        Xf, Yf = np.asfortranarray(X), np.asfortranarray(Y)
        if full:
            _lib.check(L.bse_op_eig_gradient_full(ctx.handle, a, b, bo._p(Xf), bo._p(Yf), n, NROOTS, bo._p(g),
                                                  bo._p(gm), bo._p(gh), bo._p(gw)))
        else:
            _lib.check(L.bse_op_eig_gradient(ctx.handle, 1, 2, 1, 0, bo._p(Xf), n, NROOTS, bo._p(g), bo._p(gm),
                                             bo._p(gh), bo._p(gw)))
        dX = torch.from_numpy(Xf.T.copy()).cuda()
        dY = torch.from_numpy(Yf.T.copy()).cuda()
        outs = [torch.full((NAUX * sz,), float("nan"), dtype=torch.float64, device="cuda")
                for sz in (n, n, V * V, C * C, (V + C) ** 2, 1)]
        ptr = [ctypes.c_void_p(t.data_ptr()) for t in outs]
        ptr[4] = ctypes.c_void_p(outs[4].data_ptr())
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        _lib.check(L.bse_op_eig_gradient_device(ctx.handle, a, b, ctypes.c_void_p(dX.data_ptr()),
                                                ctypes.c_void_p(dY.data_ptr()) if full else None, n, NROOTS,
                                                bo._p(g), *ptr, stream))
        vc, cv, vv, cc, hh, ww = (t.cpu().numpy() for t in outs)
        np.testing.assert_allclose(vc.reshape(NAUX, V, C), gm[:V, :, V:V + C].transpose(1, 0, 2), atol=1e-13)
        np.testing.assert_allclose(cv.reshape(NAUX, V, C), gm[V:V + C, :, :V].transpose(1, 2, 0), atol=1e-13)
        np.testing.assert_allclose(vv.reshape(NAUX, V, V), gm[:V, :, :V].transpose(1, 0, 2), atol=1e-13)
        np.testing.assert_allclose(cc.reshape(NAUX, C, C), gm[V:V + C, :, V:V + C].transpose(1, 0, 2), atol=1e-13)
        np.testing.assert_allclose(hh[:(V + C) ** 2].reshape((V + C, V + C), order="F"), gh, atol=1e-13)
        np.testing.assert_allclose(ww[:NAUX], gw, atol=1e-13)


@pytest.mark.parametrize("prec", ["mixed", "sliced"])
def test_tensor_core_adjoint_matches_fp64(prec):
    """Handles with a tensor-core engine form the two cc-block contractions of the gradient as
    FP64-accurate slice products: the same gradient as the FP64 handle to about 1e-10 of each
    block's scale (singlet and triplet coefficient sets, 4 vectors, dense enough to exercise the
    chunking of the vectors)."""
    from votca_gb300 import bse_operator as bo

    v, c, naux = 12, 80, 150
    p = Problem(v=v, c=c, naux=naux, nmo=v + c, seed=17)
    opt = bo.BSEOperator_Options(homo=v - 1, rpamin=0, qpmin=0, vmin=0, cmax=v + c - 1)
    M = bo.TCMatrix_gwbse(p.mmn)
    f = bo.GpuBSEContext(p.w, M, p.hqp, opt, precision=bo.PRECISION_FP64)
    t = bo.GpuBSEContext(p.w, M, p.hqp, opt,
                         precision=bo.PRECISION_MIXED if prec == "mixed" else bo.PRECISION_SLICED)
    rng = np.random.default_rng(3)
    X = np.asfortranarray(rng.standard_normal((v * c, 4)))
    X /= np.linalg.norm(X, axis=0)
    g = np.array([1.0, -0.5, 0.7, 0.3])
    nh = v + c
    for coef in ((1, 2, 1, 0), (1, 0, 1, 0)):
        out = []
        for ctx in (f, t):
            gm = np.zeros(p.mmn.shape)
            gh = np.zeros((nh, nh), order="F")
            gw = np.zeros(p.w.shape)
            from votca_gb300 import _lib
            _lib.check(ctx._L.bse_op_eig_gradient(ctx.handle, *coef, bo._p(X), X.shape[0], 4, bo._p(g),
                                                  bo._p(gm), bo._p(gh), bo._p(gw)))
            out.append((gm, gh, gw))
        for a, b, name in zip(out[0], out[1], ("mmn", "hqp", "w")):
            err = np.linalg.norm(b - a) / max(np.linalg.norm(a), 1e-300)
            print(f"{prec} {coef} {name}: {err:.2e}")
            assert err < 1e-9, (coef, name, err)
    f.close()
    t.close()
