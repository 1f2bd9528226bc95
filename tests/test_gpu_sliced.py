"""Ozaki slice products (BSE_PRECISION_SLICED) against the FP64 path and the oracle.

Every FP64 operand is cut into five 7-bit digit planes with a power-of-two scale per run of at
most 1024 K elements; each pair of digit levels is accumulated exactly in FP32 over one run on
the tensor cores and the runs are summed in FP64.  The products must agree with the FP64 DGEMM
path to about 1e-11 of the interaction part (the digits beyond the fifth level are dropped), far
below the 1e-5 of the BF16x3 split products.
"""
import numpy as np
import pytest

import oracle
from votca_gb300.synthetic import Problem

pytestmark = pytest.mark.gpu

# five digits of 7 bits: about 2^-36 of each run's largest element per operand and product
# term, so ~1e-10 of the product norm for Gaussian data (a run's maximum is a few times its
# typical element); measured 1.1e-10 on the C0 Hx product
SLICED_TOL = 3e-10


def contexts(p, vt, ct, voff=0):
    from votca_gb300 import bse_operator as bo

    Mmn = bo.TCMatrix_gwbse(p.mmn)
    opt = bo.BSEOperator_Options(homo=voff + vt - 1, rpamin=0, qpmin=0, vmin=voff, cmax=voff + vt + ct - 1)
    hqp = p.hqp[voff:voff + vt + ct, voff:voff + vt + ct]
    f = bo.GpuBSEContext(p.w, Mmn, hqp, opt, precision=bo.PRECISION_FP64)
    s = bo.GpuBSEContext(p.w, Mmn, hqp, opt, precision=bo.PRECISION_SLICED)
    return f, s


SHAPES = [
    (8, 64, 256, 72, 0, 0, 7),       # C0
    (3, 17, 37, 29, 2, 11, 5),       # every K padded, partial tiles
    (16, 200, 300, 216, 0, 5, 70),   # k > 64: the Hx column blocks
    (70, 40, 30, 110, 0, 6, 3),      # v > 64: the Hd stage-2 and Hd2 column blocks
    (1, 1, 5, 2, 0, 4, 2),           # degenerate
]


@pytest.mark.parametrize("v,c,naux,nmo,voff,seed,k", SHAPES)
def test_sliced_matches_fp64(v, c, naux, nmo, voff, seed, k):
    from votca_gb300 import bse_operator as bo

    p = Problem(v=v + voff, c=c, naux=naux, nmo=nmo + voff, seed=seed)
    f, s = contexts(p, v, c, voff)
    X = np.random.default_rng(seed).standard_normal((v * c, k))
    for op in ("hx", "hd", "hd2"):
        yf = bo.BSE_OPERATOR(f, *oracle.OPERATORS[op]).matmul(X)
        ys = bo.BSE_OPERATOR(s, *oracle.OPERATORS[op]).matmul(X)
        err = np.linalg.norm(ys - yf) / np.linalg.norm(yf)
        assert err < SLICED_TOL, (op, err)
    hq = bo.HqpOperator(f).matmul(X)
    for op in ("singlet", "triplet", "singlet_b"):
        yf = bo.BSE_OPERATOR(f, *oracle.OPERATORS[op]).matmul(X)
        ys = bo.BSE_OPERATOR(s, *oracle.OPERATORS[op]).matmul(X)
        inter = yf - (hq if oracle.OPERATORS[op][0] else 0)
        err = np.linalg.norm(ys - yf) / np.linalg.norm(inter)
        print(f"{op} v{v} c{c} naux{naux} k{k}: sliced vs FP64 {err:.2e}")
        assert err < SLICED_TOL, (op, err)


@pytest.mark.parametrize("v,c,naux", [
    (3, 1100, 40),   # K = c padded to 1152: digit runs of 576
    (4, 64, 2400),   # K = Naux * v = 9600: digit runs of 960
])
def test_sliced_odd_digit_runs(v, c, naux):
    """Digit runs shorter than 1024 where 1024 does not divide the padded K, against the
    oracle's factorised product."""
    from votca_gb300 import bse_operator as bo

    p = Problem(v=v, c=c, naux=naux, nmo=v + c, seed=31)
    f, s = contexts(p, v, c)
    X = np.random.default_rng(31).standard_normal((v * c, 4))
    orc = oracle.BSEProblem(p.mmn, p.w, p.hqp, v, c)
    for op in ("singlet", "singlet_b"):
        ys = bo.BSE_OPERATOR(s, *oracle.OPERATORS[op]).matmul(X)
        yo = orc.matmul_fact(X, op)
        yf = bo.BSE_OPERATOR(f, *oracle.OPERATORS[op]).matmul(X)
        hq = bo.HqpOperator(f).matmul(X) if oracle.OPERATORS[op][0] else 0
        err = np.linalg.norm(ys - yo) / np.linalg.norm(yo - hq)
        assert err < SLICED_TOL, (op, err)
        assert np.linalg.norm(yf - yo) / np.linalg.norm(yo - hq) < 1e-12


def test_sliced_full_bse_product():
    """The HAM product [[A, B], [-B, -A]] with both blocks as slice products."""
    from votca_gb300 import bse_operator as bo

    p = Problem(v=12, c=90, naux=200, nmo=102, seed=41)
    f, s = contexts(p, 12, 90)
    X = np.random.default_rng(41).standard_normal((2 * 12 * 90, 6))
    yf = bo.HamiltonianOperator(bo.SingletOperator_TDA(f), bo.SingletOperator_BTDA_B(f)).matmul(X)
    ys = bo.HamiltonianOperator(bo.SingletOperator_TDA(s), bo.SingletOperator_BTDA_B(s)).matmul(X)
    hq = np.vstack([bo.HqpOperator(f).matmul(X[:1080]), -bo.HqpOperator(f).matmul(X[1080:])])
    assert np.linalg.norm(ys - yf) / np.linalg.norm(yf - hq) < SLICED_TOL


@pytest.mark.parametrize("kind", ["singlet", "triplet"])
def test_sliced_solve_and_polish_modes(kind):
    """A SLICED solve, and a MIXED solve polished with slice products and with FP64 DGEMM
    products: the same roots as the FP64 solve to FP64 rounding of the Rayleigh quotients."""
    from votca_gb300 import bse_operator as bo
    from votca_gb300.davidson import DavidsonSolver

    cls = bo.SingletOperator_TDA if kind == "singlet" else bo.TripletOperator_TDA
    p = Problem(v=16, c=200, naux=300, nmo=216, seed=7)
    f, s = contexts(p, 16, 200)
    Mmn = bo.TCMatrix_gwbse(p.mmn)
    opt = bo.BSEOperator_Options(homo=15, rpamin=0, qpmin=0, vmin=0, cmax=215)
    m = bo.GpuBSEContext(p.w, Mmn, p.hqp, opt, precision=bo.PRECISION_MIXED)
    res = {}
    for name, ctx, pol in (("fp64", f, True), ("sliced", s, True), ("mixed_sliced", m, "sliced"),
                           ("mixed_dgemm", m, "fp64")):
        ds = DavidsonSolver()
        ds.set_tolerance(1e-8)
        ds.set_max_search_space(120)
        ds.set_fp64_polish(pol)
        lam, X = ds.solve(cls(ctx), 10)
        assert ds.info() == "Success", name
        res[name] = (lam, X, ds.result)
    assert res["sliced"][2].polished == 0  # slice products need no polish
    lam_f, Xf, _ = res["fp64"]
    for name in ("sliced", "mixed_sliced", "mixed_dgemm"):
        lam, X, r = res[name]
        R = cls(f).matmul(X) - X * lam  # residuals under the FP64 operator
        assert np.linalg.norm(R, axis=0).max() <= 1.01e-8, name
        assert np.max(np.abs(lam - lam_f)) <= 1e-10, (name, np.abs(lam - lam_f).max())
        assert np.all(np.abs(np.sum(X * Xf, axis=0)) >= 1 - 1e-10), name
    assert res["mixed_sliced"][2].polished == 1 and res["mixed_dgemm"][2].polished == 1
