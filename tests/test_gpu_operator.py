"""GPU parity of the BSE operator (FP64) against the CPU oracle, through the C ABI."""
import os

import numpy as np
import pytest

import oracle
from tests.conftest import is_approx
from votca_gb300.synthetic import Problem, dense_screening

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL = 1e-11  # FP64 vs FP64 with a different summation order (normwise relative)


def gpu_ctx(p, vt, ct, voff=0, prec=0, dense_w=None, mmin=0):
    from votca_gb300 import bse_operator as bo

    Mmn = bo.TCMatrix_gwbse(p.mmn, mmin=mmin, nmin=mmin)
    opt = bo.BSEOperator_Options(homo=mmin + voff + vt - 1, rpamin=mmin, qpmin=mmin, vmin=mmin + voff,
                                 cmax=mmin + voff + vt + ct - 1)
    hqp = p.hqp[voff:voff + vt + ct, voff:voff + vt + ct]
    return bo.GpuBSEContext(p.w, Mmn, hqp, opt, precision=prec, dense_screening=dense_w)


def oracle_prob(p, vt, ct, voff=0):
    hqp = p.hqp[voff:voff + vt + ct, voff:voff + vt + ct]
    return oracle.BSEProblem(p.mmn, p.w, hqp, vt, ct, voff=voff, coff=voff + vt)


def test_hqp_operator_matches_reference_golden():
    from votca_gb300 import bse_operator as bo

    g = np.load(os.path.join(GOLD, "bse_operator_hqp.npz"))
    Mmn = bo.TCMatrix_gwbse.Initialize(17, 0, 16, 0, 16)
    opt = bo.BSEOperator_Options(homo=4, rpamin=0, qpmin=0, vmin=0, cmax=8)
    ctx = bo.GpuBSEContext(g["epsilon_inv"], Mmn, g["Hqp"], opt)
    op = bo.HqpOperator(ctx)
    mat = op.matmul(np.eye(op.rows()))
    assert is_approx(mat, g["hqp_ref"], 1e-3)
    assert np.max(np.abs(mat - g["hqp_ref"])) < 1e-5
    assert is_approx(np.diag(mat), op.diagonal(), 1e-3)


@pytest.fixture(scope="module")
def small():
    p = Problem(v=5, c=7, naux=11, nmo=14, seed=3)
    return p, gpu_ctx(p, 5, 7), oracle_prob(p, 5, 7)


@pytest.mark.parametrize("op", list(oracle.OPERATORS))
def test_matmul_matches_oracle(small, op):
    from votca_gb300 import bse_operator as bo

    p, ctx, orc = small
    X = np.random.default_rng(7).standard_normal((orc.dim, 9))
    Y = bo.BSE_OPERATOR(ctx, *oracle.OPERATORS[op]).matmul(X)
    assert is_approx(Y, orc.matmul_ref(X, op), TOL)


@pytest.mark.parametrize("op", list(oracle.OPERATORS))
def test_diagonal_matches_oracle(small, op):
    from votca_gb300 import bse_operator as bo

    p, ctx, orc = small
    D = bo.BSE_OPERATOR(ctx, *oracle.OPERATORS[op]).diagonal()
    assert np.allclose(D, orc.diagonal(op), rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("v,c,naux,nmo,voff,seed", [(8, 64, 256, 72, 0, 0), (3, 17, 37, 29, 2, 11),
                                                     (1, 1, 5, 2, 0, 4), (6, 33, 64, 45, 4, 8)])
def test_ragged_and_offset_windows(v, c, naux, nmo, voff, seed):
    from votca_gb300 import bse_operator as bo

    p = Problem(v=v + voff, c=c, naux=naux, nmo=nmo + voff, seed=seed)
    ctx = gpu_ctx(p, v, c, voff=voff)
    orc = oracle_prob(p, v, c, voff=voff)
    X = np.random.default_rng(seed).standard_normal((orc.dim, 5))
    for op in ("singlet", "triplet", "singlet_b"):
        Y = bo.BSE_OPERATOR(ctx, *oracle.OPERATORS[op]).matmul(X)
        assert is_approx(Y, orc.matmul_fact(X, op), TOL), op
        assert np.allclose(bo.BSE_OPERATOR(ctx, *oracle.OPERATORS[op]).diagonal(), orc.diagonal(op),
                           rtol=1e-12, atol=1e-14)


def test_config0_against_reference_loop_nest():
    """C0 sizes (v8 c64 Naux256): GPU product vs the reference's row-built loop nest."""
    from votca_gb300 import bse_operator as bo

    p = Problem(v=8, c=64, naux=256, nmo=72, seed=0)
    ctx = gpu_ctx(p, 8, 64)
    orc = oracle_prob(p, 8, 64)
    X = np.random.default_rng(1).standard_normal((orc.dim, 20))
    for op in ("singlet", "triplet", "singlet_b"):
        Y = bo.BSE_OPERATOR(ctx, *oracle.OPERATORS[op]).matmul(X)
        assert is_approx(Y, orc.matmul_ref(X, op), TOL), op


def test_identity_materialisation_is_symmetric_and_composes(small):
    from votca_gb300 import bse_operator as bo

    p, ctx, orc = small
    eye = np.eye(orc.dim)
    m = {op: bo.BSE_OPERATOR(ctx, *oracle.OPERATORS[op]).matmul(eye) for op in oracle.OPERATORS}
    assert np.allclose(m["singlet"], m["hqp"] + 2 * m["hx"] + m["hd"], atol=1e-13)
    assert np.allclose(m["singlet_b"], 2 * m["hx"] + m["hd2"], atol=1e-13)
    for a in m.values():
        assert np.allclose(a, a.T, atol=1e-13)


def test_hamiltonian_operator_block_structure(small):
    from votca_gb300 import bse_operator as bo

    p, ctx, orc = small
    A = bo.SingletOperator_TDA(ctx)
    B = bo.SingletOperator_BTDA_B(ctx)
    H = bo.HamiltonianOperator(A, B)
    X = np.random.default_rng(2).standard_normal((2 * orc.dim, 4))
    assert is_approx(H.matmul(X), orc.ham_matmul(X), TOL)
    Hm = H.matmul(np.eye(2 * orc.dim))
    Am, Bm = A.matmul(np.eye(orc.dim)), B.matmul(np.eye(orc.dim))
    assert is_approx(Hm, np.block([[Am, Bm], [-Bm, -Am]]), 1e-9)


def test_dense_screening_equals_rotated_diagonal_screening():
    """Dense W = I - eps^-1 folded at staging == reference convention (M.Q, w = 1 - 1/lambda)."""
    p = Problem(v=4, c=9, naux=24, nmo=13, seed=21)
    eps, Q, lam = dense_screening(21, 24)
    W = np.eye(24) - np.linalg.inv(eps)
    ctx = gpu_ctx(p, 4, 9, dense_w=W)
    rot = np.einsum("mpn,pq->mqn", p.mmn, Q)
    orc = oracle.BSEProblem(rot, 1.0 - 1.0 / lam, p.hqp, 4, 9)
    from votca_gb300 import bse_operator as bo

    X = np.random.default_rng(3).standard_normal((36, 6))
    for op in ("singlet", "triplet", "singlet_b", "hd", "hd2"):
        Y = bo.BSE_OPERATOR(ctx, *oracle.OPERATORS[op]).matmul(X)
        assert is_approx(Y, orc.matmul_ref(X, op), 1e-10), op
        assert np.allclose(bo.BSE_OPERATOR(ctx, *oracle.OPERATORS[op]).diagonal(), orc.diagonal(op),
                           rtol=1e-10, atol=1e-13), op


def test_zero_columns_and_bad_shapes(small):
    from votca_gb300 import bse_operator as bo
    from votca_gb300._lib import BSEError

    p, ctx, orc = small
    op = bo.SingletOperator_TDA(ctx)
    assert op.matmul(np.zeros((orc.dim, 0))).shape == (orc.dim, 0)
    with pytest.raises(BSEError):
        op.matmul(np.zeros((orc.dim + 1, 2)))


def test_repeat_is_bitwise_deterministic(small):
    from votca_gb300 import bse_operator as bo

    p, ctx, orc = small
    X = np.random.default_rng(5).standard_normal((orc.dim, 7))
    op = bo.SingletOperator_TDA(ctx)
    a = op.matmul(X)
    b = op.matmul(X)
    assert np.array_equal(a, b)
