"""Unrestricted BSE operator (BSE_OPERATOR_UKS) on the GPU through the C ABI, against the
restated reference loops (oracle/uks_oracle.py): products of every preset, diagonals,
HAM products, TDA and full-BSE roots, split precision, and the error paths."""
import numpy as np
import pytest

from oracle.uks_oracle import UKS_OPERATORS, UKSProblem as Oracle, full_bse_dense_roots
from votca_gb300.synthetic import UKSProblem

pytestmark = pytest.mark.gpu

PRESETS = {
    "tda": "ExcitonUKSOperator_TDA",
    "btda_b": "ExcitonUKSOperator_BTDA_B",
    "hd": "HdUKSOperator",
    "hd2": "Hd2UKSOperator",
    "qp": "QpUKSOperator",
    "hx": "HxUKSOperator",
}


def _setup(p, precision=0, rpamin=0):
    from votca_gb300 import bse_operator as bo
    from votca_gb300 import bse_operator_uks as bu

    mm = bu.TCMatrix_gwbse_spin(bo.TCMatrix_gwbse(p.mmn_alpha, mmin=rpamin, nmin=rpamin),
                                bo.TCMatrix_gwbse(p.mmn_beta, mmin=rpamin, nmin=rpamin))
    opt = bu.BSEOperatorUKS_Options(homo_alpha=p.homo_alpha + rpamin, homo_beta=p.homo_beta + rpamin,
                                    rpamin=rpamin, qpmin=rpamin, vmin=p.vmin + rpamin, cmax=p.cmax + rpamin)
    ctx = bu.GpuBSEContextUKS(p.w, mm, p.hqp_alpha, p.hqp_beta, opt, precision=precision)
    orc = Oracle(p.mmn_alpha, p.mmn_beta, p.w, p.hqp_alpha, p.hqp_beta, p.homo_alpha, p.homo_beta, 0, p.vmin,
                 p.cmax)
    return ctx, orc


def _op(ctx, name):
    from votca_gb300 import bse_operator_uks as bu

    return getattr(bu, PRESETS[name])(ctx)


@pytest.mark.parametrize("homos", [(6, 3), (3, 6), (4, 4)], ids=["a>b", "a<b", "a=b"])
@pytest.mark.parametrize("name", list(PRESETS))
def test_products_and_diagonals_match_reference_loops(homos, name):
    # (m, n)-asymmetric Mmn: every product must read the same M(m, n) as the reference
    p = UKSProblem(homos[0], homos[1], vmin=1, cmax=13, naux=19, nmo=16, seed=11, symmetric=False)
    ctx, orc = _setup(p, rpamin=2)
    op = _op(ctx, name)
    assert op.rows() == orc.size
    X = np.random.default_rng(1).standard_normal((orc.size, 5))
    Y = op.matmul(X)
    R = orc.matmul(X, name)
    assert np.linalg.norm(Y - R) <= 1e-12 * np.linalg.norm(R)
    np.testing.assert_allclose(op.diagonal(), orc.diagonal(name), rtol=1e-12, atol=1e-14)
    ctx.close()


@pytest.mark.parametrize("homos", [(5, 0), (0, 5), (5, 12)], ids=["beta_no_occupied", "alpha_no_occupied",
                                                               "beta_no_virtual"])
def test_empty_spin_channel(homos):
    """A spin channel without occupied (homo = vmin - 1) or without virtual (homo = cmax) levels
    in the BSE window carries an empty block (setup_block, bse_operator_uks.cc:25-35): every
    preset's product and diagonal match the restated loops, a split-precision handle agrees with
    FP64, and the TDA roots are those of the dense operator."""
    from votca_gb300 import bse_operator_uks as bu
    from votca_gb300.davidson import DavidsonSolver

    p = UKSProblem(homos[0], homos[1], vmin=1, cmax=12, naux=17, nmo=15, seed=21)
    ctx, orc = _setup(p)
    assert ctx.size == orc.size == max(orc.alpha.size, orc.beta.size) > 0
    X = np.random.default_rng(3).standard_normal((orc.size, 4))
    for name in PRESETS:
        op = _op(ctx, name)
        R = orc.matmul(X, name)
        Y = op.matmul(X)
        assert np.linalg.norm(Y - R) <= 1e-12 * np.linalg.norm(R), name
        np.testing.assert_allclose(op.diagonal(), orc.diagonal(name), rtol=1e-12, atol=1e-14)
    ctxm, _ = _setup(p, precision=1)
    Ym = _op(ctxm, "tda").matmul(X)
    Yf = orc.matmul(X, "tda")
    assert np.linalg.norm(Ym - Yf) <= 2e-4 * np.linalg.norm(Yf - orc.matmul(X, "qp"))
    ds = DavidsonSolver()
    ds.set_tolerance(1e-9)
    lam, _ = ds.solve(bu.ExcitonUKSOperator_TDA(ctx), 3)
    assert np.max(np.abs(lam - np.linalg.eigvalsh(orc.dense("tda"))[:3])) < 1e-9
    ctx.close()
    ctxm.close()


def test_ham_product_and_dense_matrix():
    from votca_gb300 import bse_operator as bo

    p = UKSProblem(5, 3, vmin=0, cmax=12, naux=17, nmo=14, seed=3, symmetric=False)
    ctx, orc = _setup(p)
    A, B = _op(ctx, "tda"), _op(ctx, "btda_b")
    Ad, Bd = orc.dense("tda"), orc.dense("btda_b")
    np.testing.assert_allclose(A.dense_matrix(), Ad, rtol=0, atol=1e-12 * np.abs(Ad).max())
    H = np.block([[Ad, Bd], [-Bd, -Ad]])
    X = np.random.default_rng(2).standard_normal((2 * orc.size, 3))
    Y = bo.HamiltonianOperator(A, B).matmul(X)
    assert np.linalg.norm(Y - H @ X) <= 1e-12 * np.linalg.norm(H @ X)
    ctx.close()


def test_tda_roots_match_dense_eigenvalues():
    from votca_gb300.bse import DavidsonOptions
    from votca_gb300.bse_operator_uks import solve_excitons_uks_tda

    p = UKSProblem(7, 5, vmin=0, cmax=40, naux=48, nmo=44, seed=6)
    ctx, orc = _setup(p)
    lam, X, ds = solve_excitons_uks_tda(ctx, DavidsonOptions(davidson_tolerance=1e-10, nmax=6))
    assert ds.info() == "Success"
    exact, vec = np.linalg.eigh(orc.dense("tda"))
    np.testing.assert_allclose(lam, exact[:6], rtol=0, atol=1e-9)
    # eigenvectors up to sign
    ov = np.abs(np.sum(X * vec[:, :6], axis=0))
    np.testing.assert_allclose(ov, 1.0, atol=1e-6)
    ctx.close()


@pytest.mark.parametrize("dims", ["dense", "davidson"])
def test_full_bse_roots(dims):
    """Solve_excitons_uks_BTDA: the dense branch (dim <= 128) and the HAM Davidson branch
    against the positive real roots of the oracle's [[A, B], [-B, -A]]."""
    from votca_gb300.bse import DavidsonOptions
    from votca_gb300.bse_operator_uks import solve_excitons_uks_btda

    if dims == "dense":
        p = UKSProblem(4, 3, vmin=0, cmax=16, naux=24, nmo=20, seed=9)   # dim 5*12 + 4*13 = 112
    else:
        p = UKSProblem(6, 4, vmin=0, cmax=36, naux=40, nmo=40, seed=9)
    ctx, orc = _setup(p)
    lam, X, Y, ds = solve_excitons_uks_btda(ctx, DavidsonOptions(davidson_tolerance=1e-10, nmax=4))
    assert (ds is None) == (orc.size <= 128)
    if ds is not None:
        assert ds.info() == "Success"
    ref, Xr, Yr = full_bse_dense_roots(orc.dense("tda"), orc.dense("btda_b"), 4)
    np.testing.assert_allclose(lam, ref, rtol=0, atol=1e-9)
    norms = np.sum(X * X, axis=0) - np.sum(Y * Y, axis=0)
    np.testing.assert_allclose(norms, 1.0, atol=1e-9)
    ctx.close()


def test_mixed_precision_products():
    p = UKSProblem(9, 6, vmin=0, cmax=70, naux=96, nmo=76, seed=12)
    ctx64, orc = _setup(p, precision=0)
    ctxm, _ = _setup(p, precision=1)
    X = np.random.default_rng(4).standard_normal((orc.size, 7))
    for name in ("tda", "btda_b", "hd"):
        Yf = _op(ctx64, name).matmul(X)
        Ym = _op(ctxm, name).matmul(X)
        inter = Yf - _op(ctx64, "qp").matmul(X) * (UKS_OPERATORS[name][0])
        assert np.linalg.norm(Ym - Yf) <= 2e-4 * np.linalg.norm(inter), name
    ctx64.close()
    ctxm.close()


def test_errors():
    from votca_gb300 import _lib
    from votca_gb300 import bse_operator as bo
    from votca_gb300 import bse_operator_uks as bu

    p = UKSProblem(4, 3, vmin=0, cmax=10, naux=9, nmo=12, seed=1)
    mm = bu.TCMatrix_gwbse_spin(bo.TCMatrix_gwbse(p.mmn_alpha), bo.TCMatrix_gwbse(p.mmn_beta[:, :8, :]))
    opt = bu.BSEOperatorUKS_Options(4, 3, 0, 0, 0, 10)
    with pytest.raises(_lib.BSEError) as e:  # different auxiliary basis sizes
        bu.GpuBSEContextUKS(p.w, mm, p.hqp_alpha, p.hqp_beta, opt)
    assert e.value.code == 1
    ctx, _ = _setup(p)
    with pytest.raises(_lib.BSEError) as e:  # both spin channels without a BSE block
        bu.GpuBSEContextUKS(p.w, bu.TCMatrix_gwbse_spin(bo.TCMatrix_gwbse(p.mmn_alpha), bo.TCMatrix_gwbse(p.mmn_beta)),
                            p.hqp_alpha, p.hqp_beta, bu.BSEOperatorUKS_Options(-1, 10, 0, 0, 0, 10))
    assert e.value.code == 1
    with pytest.raises(_lib.BSEError):  # Hd and Hd2 together
        bu.BSE_OPERATOR_UKS(ctx, 1, 1, 1, 1)
    with pytest.raises(_lib.BSEError):  # the allocation-free product is for restricted operators
        L = ctx._L
        _lib.check(L.bse_op_matmul_device_noalloc(ctx.handle, 1, 1, 1, 0, None, ctx.size, 1, None, ctx.size, None))
    ctx.close()


def test_batched_uks_solves():
    """UKS handles in the batched driver: independent solves on host threads agree with single
    solves; the lockstep mode takes restricted operators only."""
    from votca_gb300 import _lib
    from votca_gb300.bse_operator_uks import ExcitonUKSOperator_TDA
    from votca_gb300.davidson import DavidsonSolver

    ctxs = [_setup(UKSProblem(5, 3, vmin=0, cmax=30, naux=36, nmo=34, seed=s))[0] for s in (31, 32)]
    ops = [ExcitonUKSOperator_TDA(c) for c in ctxs]
    ds = DavidsonSolver()
    ds.set_tolerance(1e-9)
    ds.set_max_search_space(40)
    ev, info, _ = ds.solve_batch(ops, 4, nthreads=2)
    assert info == ["Success", "Success"]
    for m, op in enumerate(ops):
        lam, _ = _single(op)
        np.testing.assert_allclose(ev[m], lam, rtol=0, atol=1e-10)
    with pytest.raises(_lib.BSEError):
        ds.solve_batch(ops, 4, nthreads=0)
    for c in ctxs:
        c.close()


def _single(op):
    from votca_gb300.davidson import DavidsonSolver

    ds = DavidsonSolver()
    ds.set_tolerance(1e-9)
    ds.set_max_search_space(40)
    return ds.solve(op, 4)
