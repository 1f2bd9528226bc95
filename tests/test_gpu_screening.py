"""Screening on the GPU: RPA epsilon, Cholesky inverse, MultiplyRightWithAuxMatrix,
and the dense-screening operator against the reference's rotate-and-invert convention."""
import ctypes

import numpy as np
import pytest

import oracle
from oracle.rpa_oracle import epsilon_r, setup_screening
from tests.conftest import is_approx
from votca_gb300.synthetic import Problem

pytestmark = pytest.mark.gpu


def _desc_ptrs(mmn, mmin=0):
    from votca_gb300 import _lib

    desc = _lib.bse_mmn_desc(mmn.shape[1], mmin, mmin + mmn.shape[0] - 1, mmin, mmin + mmn.shape[2] - 1)
    ptrs = (_lib.c_dp * mmn.shape[0])(*[ctypes.cast(mmn.ctypes.data + m * mmn.strides[0], _lib.c_dp)
                                        for m in range(mmn.shape[0])])
    return desc, ptrs


def _p(a):
    from votca_gb300 import _lib

    return a.ctypes.data_as(_lib.c_dp)


@pytest.mark.parametrize("freq", [0.0 + 0.0j, 0.3 + 0.0j, 0.0 + 0.5j])
def test_rpa_epsilon_matches_oracle(freq):
    from votca_gb300 import _lib

    L = _lib.load()
    p = Problem(v=6, c=30, naux=40, nmo=44, seed=2)  # rpamax beyond the BSE window
    energies = np.concatenate([np.diag(p.hqp), np.linspace(31, 40, 44 - 36)])
    homo, rpamin, rpamax = 5, 0, 43
    eps = np.zeros((40, 40), order="F")
    desc, ptrs = _desc_ptrs(p.mmn)
    _lib.check(L.bse_rpa_epsilon(ctypes.byref(desc), ptrs, _p(energies), 44, homo, rpamin, rpamax,
                                 freq.real, freq.imag, _p(eps)))
    ref = epsilon_r(p.mmn, energies, homo, rpamin, rpamax, freq)
    assert np.allclose(eps, ref, rtol=1e-12, atol=1e-13)


@pytest.mark.parametrize("n", [1, 7, 64, 100, 257])
def test_cholesky_inverse(n):
    from votca_gb300 import _lib

    L = _lib.load()
    rng = np.random.default_rng(n)
    G = rng.standard_normal((n, n))
    A = np.asfortranarray(G @ G.T + n * np.eye(n))
    Ai = np.zeros((n, n), order="F")
    _lib.check(L.bse_cholesky_inverse(n, _p(A), n, _p(Ai), n))
    assert np.allclose(Ai @ A, np.eye(n), atol=1e-10)
    assert np.allclose(Ai, np.linalg.inv(A), rtol=1e-10, atol=1e-12)


def test_cholesky_rejects_indefinite():
    from votca_gb300 import _lib

    L = _lib.load()
    A = np.asfortranarray(np.diag([1.0, -2.0, 3.0]))
    Ai = np.zeros((3, 3), order="F")
    rc = L.bse_cholesky_inverse(3, _p(A), 3, _p(Ai), 3)
    assert rc == 5 and b"positive definite" in L.bse_last_error()


def test_positive_inverse_drops_small_and_negative_modes():
    """The reference's screening for any symmetric eps: modes with lambda <= 1e-8 dropped."""
    from votca_gb300.screening import positive_inverse

    rng = np.random.default_rng(7)
    Q, _ = np.linalg.qr(rng.standard_normal((50, 50)))
    # kept modes well above the cutoff and dropped modes well below it (an eigenvalue next to
    # the cutoff would make 1/lambda depend on rounding)
    lam = np.concatenate([np.linspace(0.5, 4.0, 45), [-0.3, -1e-3, 0.0, 1e-10, -1e-10]])
    A = (Q * lam) @ Q.T
    A = 0.5 * (A + A.T)
    W = positive_inverse(A, 1e-8)
    lam_n, U = np.linalg.eigh(A)
    w = np.where(lam_n > 1e-8, 1.0 / np.where(lam_n > 1e-8, lam_n, 1.0), 0.0)
    assert np.allclose(W, (U * w) @ U.T, rtol=1e-10, atol=1e-12)
    assert np.linalg.matrix_rank(W, tol=1e-8) == 45


def test_multiply_right_with_aux_matrix():
    from votca_gb300 import _lib

    L = _lib.load()
    p = Problem(v=3, c=9, naux=17, nmo=12, seed=4)
    m = p.mmn.copy()
    U = np.asfortranarray(np.random.default_rng(3).standard_normal((17, 17)))
    desc, ptrs = _desc_ptrs(m)
    _lib.check(L.bse_mmn_multiply_right(ctypes.byref(desc), ptrs, _p(U), 17))
    ref = np.einsum("mpn,pq->mqn", p.mmn, U)
    assert np.allclose(m, ref, rtol=1e-12, atol=1e-14)


def test_screened_operator_rpa_cholesky_route_equals_reference_convention():
    """RPA eps -> GPU Cholesky inverse -> dense screening operator == reference
    SetupDirectInteractionOperator (eigenvectors rotate Mmn, w = 1/lambda)."""
    from votca_gb300 import _lib
    from votca_gb300 import bse_operator as bo

    L = _lib.load()
    p = Problem(v=5, c=20, naux=30, nmo=25, seed=9)
    energies = np.diag(p.hqp).copy()
    eps = np.zeros((30, 30), order="F")
    desc, ptrs = _desc_ptrs(p.mmn)
    _lib.check(L.bse_rpa_epsilon(ctypes.byref(desc), ptrs, _p(energies), 25, 4, 0, 24, 0.0, 0.0, _p(eps)))
    W = np.zeros((30, 30), order="F")
    _lib.check(L.bse_cholesky_inverse(30, _p(eps), 30, _p(W), 30))
    opt = bo.BSEOperator_Options(homo=4, rpamin=0, qpmin=0, vmin=0, cmax=24)
    ctx = bo.GpuBSEContext(None, bo.TCMatrix_gwbse(p.mmn), p.hqp, opt, dense_screening=W)
    rot, w = setup_screening(p.mmn, epsilon_r(p.mmn, energies, 4, 0, 24))
    orc = oracle.BSEProblem(rot, w, p.hqp, 5, 20)
    X = np.random.default_rng(0).standard_normal((100, 4))
    for op in ("singlet", "triplet", "hd"):
        assert is_approx(bo.BSE_OPERATOR(ctx, *oracle.OPERATORS[op]).matmul(X), orc.matmul_ref(X, op), 1e-10)
