"""FP64 polish of split-precision Davidson solves, and the block-size / initial-size options.

The polish (no counterpart in the reference) re-applies the converged Ritz vectors with FP64
products and iterates on that basis until the residuals, formed from FP64 products, meet the
tolerance: the returned roots must then satisfy the FP64 operator to the tolerance and agree
with an FP64 solve to FP64 rounding of the Rayleigh quotients.
"""
import numpy as np
import pytest

import oracle
from votca_gb300.synthetic import Problem

pytestmark = pytest.mark.gpu


def _contexts(p, v, c):
    from votca_gb300 import bse_operator as bo

    Mmn = bo.TCMatrix_gwbse(p.mmn)
    opt = bo.BSEOperator_Options(homo=v - 1, rpamin=0, qpmin=0, vmin=0, cmax=v + c - 1)
    f = bo.GpuBSEContext(p.w, Mmn, p.hqp, opt, precision=bo.PRECISION_FP64)
    m = bo.GpuBSEContext(p.w, Mmn, p.hqp, opt, precision=bo.PRECISION_MIXED)
    return f, m


@pytest.mark.parametrize("kind", ["singlet", "triplet"])
def test_tda_polish_reaches_fp64_residuals(kind):
    from votca_gb300 import bse_operator as bo
    from votca_gb300.davidson import DavidsonSolver

    cls = bo.SingletOperator_TDA if kind == "singlet" else bo.TripletOperator_TDA
    p = Problem(v=16, c=200, naux=300, nmo=216, seed=5)
    f, m = _contexts(p, 16, 200)
    res = {}
    for name, ctx, pol in (("fp64", f, True), ("mixed", m, True), ("raw", m, False)):
        ds = DavidsonSolver()
        ds.set_tolerance(1e-8 if pol else 1e-6)  # the split products alone stall near 1e-7
        ds.set_max_search_space(120)
        ds.set_fp64_polish(pol)
        lam, X = ds.solve(cls(ctx), 12)
        assert ds.info() == "Success", name
        res[name] = (lam, X, ds.result)
    assert res["fp64"][2].polished == 0 and res["fp64"][2].fp64_columns == 0  # nothing to polish
    assert res["raw"][2].polished == 0
    r = res["mixed"][2]
    assert r.polished == 1 and r.fp64_columns >= 12 and r.polish_iterations >= 1
    lam_m, Xm, _ = res["mixed"]
    lam_f, Xf, _ = res["fp64"]
    # residuals under the FP64 operator and under the oracle's product
    R = cls(f).matmul(Xm) - Xm * lam_m
    assert np.linalg.norm(R, axis=0).max() <= 1e-8
    orc = oracle.BSEProblem(p.mmn, p.w, p.hqp, 16, 200)
    Ro = orc.matmul_fact(Xm, kind) - Xm * lam_m
    assert np.linalg.norm(Ro, axis=0).max() <= 1.01e-8
    assert r.max_residual <= 1e-8
    # polished Rayleigh quotients agree with the FP64 solve far below the split error
    assert np.max(np.abs(lam_m - lam_f)) <= 1e-10, np.abs(lam_m - lam_f)
    assert np.all(np.abs(np.sum(Xm * Xf, axis=0)) >= 1 - 1e-10)
    # the unpolished split solve is only as good as the split products
    assert np.max(np.abs(res["raw"][0] - lam_f)) < 1e-5


def test_full_bse_polish_against_dense_eig():
    """HAM polish: the projected pencil (V^T S V, V^T J V) of [[A, B], [-B, -A]] = J S."""
    from votca_gb300 import bse_operator as bo
    from votca_gb300.bse import DavidsonOptions, solve_nonhermitian_davidson

    p = Problem(v=6, c=40, naux=96, nmo=46, seed=12)
    f, m = _contexts(p, 6, 40)
    orc = oracle.BSEProblem(p.mmn, p.w, p.hqp, 6, 40)
    A, B = orc.dense("singlet"), orc.dense("singlet_b")
    H = np.block([[A, B], [-B, -A]])
    ev = np.linalg.eigvals(H).real
    ref = np.sort(ev[ev > 0])[:6]
    lam, X, Y, ds = solve_nonhermitian_davidson(bo.SingletOperator_TDA(m), bo.SingletOperator_BTDA_B(m),
                                                DavidsonOptions(davidson_tolerance=1e-8, nmax=6))
    assert ds.info() == "Success" and ds.result.polished == 1
    assert np.max(np.abs(np.sort(lam) - ref)) < 1e-10
    Z = np.vstack([X, Y])
    assert np.linalg.norm(H @ Z - Z * lam, axis=0).max() <= 1e-8 * np.linalg.norm(Z, axis=0).max()
    assert np.allclose(np.sum(X * X, axis=0) - np.sum(Y * Y, axis=0), 1.0, atol=1e-10)


def test_block_size_and_initial_size():
    """set_block_size (trial vectors per iteration) and set_initial_size (the size_initial_guess
    overload): same roots as the reference's defaults; errors below neigen."""
    from votca_gb300 import _lib
    from votca_gb300 import bse_operator as bo
    from votca_gb300.davidson import DavidsonSolver

    p = Problem(v=8, c=64, naux=256, nmo=72, seed=0)
    f, _ = _contexts(p, 8, 64)
    op = bo.SingletOperator_TDA(f)
    ref = np.linalg.eigvalsh(oracle.BSEProblem(p.mmn, p.w, p.hqp, 8, 64).dense("singlet"))[:10]
    for block, init in ((0, 0), (32, 0), (12, 25), (32, 32)):
        ds = DavidsonSolver()
        ds.set_tolerance(1e-9)
        ds.set_max_search_space(100)
        ds.set_block_size(block)
        ds.set_initial_size(init)
        lam, _ = ds.solve(op, 10)
        assert ds.info() == "Success", (block, init)
        assert np.max(np.abs(lam - ref)) < 1e-9, (block, init)
        if block == 32 and init == 32:
            assert ds.result.matvec_columns >= 32 + 32 or ds.num_iterations() == 0
    for block, init in ((5, 0), (0, 7)):
        ds = DavidsonSolver()
        ds.set_block_size(block)
        ds.set_initial_size(init)
        with pytest.raises(_lib.BSEError):
            ds.solve(op, 10)
