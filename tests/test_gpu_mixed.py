"""Mixed-precision (tcgen05 BF16x3) BSE product and solve against the FP64 path."""
import numpy as np
import pytest

import oracle
from votca_gb300.synthetic import Problem

pytestmark = pytest.mark.gpu

# BF16x3 split products with FP32 accumulation: ~1e-5 relative on the
# interaction part of the product (Hx, Hd, Hd2; measured 0.5-1.2e-5 on these shapes and at the
# headline size); Hqp is exact FP64.  A few times the measured error, so that a regression of the
# split arithmetic (a dropped product, a longer FP32 chain) fails.
REL_TOL = 5e-5


def contexts(p, vt, ct, voff=0):
    from votca_gb300 import bse_operator as bo

    Mmn = bo.TCMatrix_gwbse(p.mmn)
    opt = bo.BSEOperator_Options(homo=voff + vt - 1, rpamin=0, qpmin=0, vmin=voff, cmax=voff + vt + ct - 1)
    hqp = p.hqp[voff:voff + vt + ct, voff:voff + vt + ct]
    f = bo.GpuBSEContext(p.w, Mmn, hqp, opt, precision=bo.PRECISION_FP64)
    m = bo.GpuBSEContext(p.w, Mmn, hqp, opt, precision=bo.PRECISION_MIXED)
    return f, m


SHAPES = [
    (8, 64, 256, 72, 0, 0),     # C0
    (3, 17, 37, 29, 2, 11),     # everything ragged (padding of K, partial tiles)
    (6, 33, 64, 45, 4, 8),
    (16, 200, 300, 216, 0, 5),  # several N tiles, K split
    (1, 1, 5, 2, 0, 4),         # degenerate
]


@pytest.mark.parametrize("v,c,naux,nmo,voff,seed", SHAPES)
def test_mixed_matches_fp64(v, c, naux, nmo, voff, seed):
    from votca_gb300 import bse_operator as bo

    p = Problem(v=v + voff, c=c, naux=naux, nmo=nmo + voff, seed=seed)
    f, m = contexts(p, v, c, voff)
    X = np.random.default_rng(seed).standard_normal((v * c, 7))
    for op in ("hx", "hd", "hd2"):
        yf = bo.BSE_OPERATOR(f, *oracle.OPERATORS[op]).matmul(X)
        ym = bo.BSE_OPERATOR(m, *oracle.OPERATORS[op]).matmul(X)
        err = np.linalg.norm(ym - yf) / np.linalg.norm(yf)
        print(f"mixed {op}: {err:.2e}")
        assert err < REL_TOL, (op, err)
    hq = bo.HqpOperator(f).matmul(X)
    for op in ("singlet", "triplet", "singlet_b"):
        yf = bo.BSE_OPERATOR(f, *oracle.OPERATORS[op]).matmul(X)
        ym = bo.BSE_OPERATOR(m, *oracle.OPERATORS[op]).matmul(X)
        inter = yf - (hq if oracle.OPERATORS[op][0] else 0)
        err = np.linalg.norm(ym - yf) / np.linalg.norm(inter)
        print(f"mixed {op}: {err:.2e}")
        assert err < REL_TOL, (op, err)


def test_mixed_many_vectors_chunked():
    """k = 37 vectors (not a multiple of any tile), two vectors per intermediate chunk."""
    from votca_gb300 import bse_operator as bo

    p = Problem(v=8, c=64, naux=256, nmo=72, seed=2)
    f, m = contexts(p, 8, 64)
    X = np.random.default_rng(3).standard_normal((512, 37))
    yf = bo.SingletOperator_TDA(f).matmul(X)
    ym = bo.SingletOperator_TDA(m).matmul(X)
    inter = yf - bo.HqpOperator(f).matmul(X)
    assert np.linalg.norm(ym - yf) / np.linalg.norm(inter) < REL_TOL


@pytest.mark.parametrize("v,c,naux,seed", [
    (5, 200, 700, 21),   # ragged K of the Hd2 stage-2 chain (naux * v = 3500)
    (20, 64, 3000, 22),  # long aux chains (K = 60000 split into chains of <= 1024)
])
def test_mixed_long_aux_products(v, c, naux, seed):
    """Products with many aux functions per (v, c) pair, 30 vectors."""
    from votca_gb300 import bse_operator as bo

    p = Problem(v=v, c=c, naux=naux, nmo=v + c, seed=seed)
    f, m = contexts(p, v, c)
    X = np.random.default_rng(seed).standard_normal((v * c, 30))
    hq = bo.HqpOperator(f).matmul(X)
    for op in ("hd", "hd2", "singlet", "singlet_b"):
        yf = bo.BSE_OPERATOR(f, *oracle.OPERATORS[op]).matmul(X)
        ym = bo.BSE_OPERATOR(m, *oracle.OPERATORS[op]).matmul(X)
        inter = yf - (hq if oracle.OPERATORS[op][0] else 0)
        err = np.linalg.norm(ym - yf) / np.linalg.norm(inter)
        print(f"mixed {op}: {err:.2e}")
        assert err < REL_TOL, (op, err)


def test_mixed_davidson_roots_within_tolerance():
    """C0 singlets and triplets, 10 roots at residual 1e-7: every root within 0.01 meV of FP64."""
    from votca_gb300 import bse_operator as bo
    from votca_gb300.davidson import DavidsonSolver

    p = Problem(v=8, c=64, naux=256, nmo=72, seed=0)
    f, m = contexts(p, 8, 64)
    for cls in (bo.SingletOperator_TDA, bo.TripletOperator_TDA):
        res = []
        for ctx in (f, m):
            ds = DavidsonSolver()
            ds.set_tolerance(1e-7)
            ds.set_max_search_space(100)
            lam, vec = ds.solve(cls(ctx), 10)
            assert ds.info() == "Success"
            res.append((lam, vec))
        dmev = np.abs(res[0][0] - res[1][0]) * 1e3
        assert dmev.max() < 0.01, dmev
        ov = np.abs(np.sum(res[0][1] * res[1][1], axis=0))
        assert np.all(ov > 1 - 1e-6)
