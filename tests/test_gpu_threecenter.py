"""Mmn producer on the GPU (TCMatrix_gwbse::Fill3cMO with caller integrals,
AOCoulomb::Pseudo_InvSqrt(_GWBSE), TCMatrix_gwbse::Fill) through the C ABI, against the
oracle and the reference's golden auxiliary-metric matrices."""
import os

import numpy as np
import pytest

from oracle.threecenter_oracle import fill_3c_mo as fill_ref, pseudo_inv_sqrt as pis_ref
from oracle.threecenter_oracle import pseudo_inv_sqrt_gwbse as pisgw_ref
from tests.conftest import is_approx

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _ao_problem(naux, nbf, nmo, seed):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((naux, nbf, nbf)) * 0.3
    A = A + A.transpose(0, 2, 1)
    C = rng.standard_normal((nbf, nmo)) / np.sqrt(nbf)
    return A, C


def test_aux_metric_against_golden_and_oracle():
    from votca_gb300 import threecenter as tc

    g = np.load(os.path.join(GOLD, "aomatrix.npz"))
    m, removed = tc.pseudo_inv_sqrt(g["coulomb"], 1e-7)
    assert removed == 0 and is_approx(m, g["invsqrt"], 5e-4)  # 6-digit golden inputs, cond(V) ~ 1.3e3
    np.testing.assert_allclose(m, pis_ref(g["coulomb"], 1e-7)[0], rtol=0, atol=1e-11)
    mg, removed = tc.pseudo_inv_sqrt_gwbse(g["overlap"], g["coulomb"], 1e-7)
    assert removed == 0 and is_approx(mg, g["invsqrt_gwbse"], 5e-4)
    np.testing.assert_allclose(mg, pisgw_ref(g["overlap"], g["coulomb"], 1e-7)[0], rtol=0, atol=1e-11)


def test_aux_metric_removes_small_eigenvalues():
    from votca_gb300 import threecenter as tc

    rng = np.random.default_rng(3)
    Q, _ = np.linalg.qr(rng.standard_normal((40, 40)))
    lam = np.concatenate([[1e-9, 3e-8], np.linspace(0.2, 5.0, 38)])
    V = (Q * lam) @ Q.T
    S = np.eye(40) + 0.05 * (lambda B: B + B.T)(rng.standard_normal((40, 40))) / 10
    m, r = tc.pseudo_inv_sqrt(V, 5e-7)
    mr, rr = pis_ref(V, 5e-7)
    assert r == rr == 2
    np.testing.assert_allclose(m, mr, rtol=0, atol=1e-9)
    mg, rg = tc.pseudo_inv_sqrt_gwbse(S, V, 5e-7)
    mgr, rgr = pisgw_ref(S, V, 5e-7)
    assert rg == rgr
    np.testing.assert_allclose(mg, mgr, rtol=0, atol=1e-8 * np.abs(mgr).max())


@pytest.mark.parametrize("max_p", [None, 7])
def test_fill_3c_mo_matches_oracle(monkeypatch, max_p):
    from votca_gb300 import bse_operator as bo
    from votca_gb300 import threecenter as tc

    if max_p is not None:  # several auxiliary chunks (ragged last chunk)
        monkeypatch.setenv("VGB_FILL3C_MAX_P", str(max_p))
    naux, nbf, nmo = 37, 29, 25
    A, C = _ao_problem(naux, nbf, nmo, 1)
    M = bo.TCMatrix_gwbse.Initialize(naux, 2, 20, 0, 24)
    tc.fill_3c_mo(M, A, C)
    R = fill_ref(A, C, 2, 20, 0, 24)
    assert np.linalg.norm(M.data - R) <= 1e-13 * np.linalg.norm(R)


def test_fill_chain_feeds_the_operator():
    """TCMatrix_gwbse::Fill (Fill3cMO, then the GW-BSE metric) and a BSE product built on the
    result, against the oracle chain and the RKS oracle operator."""
    import oracle
    from votca_gb300 import bse_operator as bo
    from votca_gb300 import threecenter as tc

    naux, nbf, nmo = 24, 30, 22
    A, C = _ao_problem(naux, nbf, nmo, 5)
    rng = np.random.default_rng(6)
    Q, _ = np.linalg.qr(rng.standard_normal((naux, naux)))
    V = (Q * np.linspace(0.5, 4.0, naux)) @ Q.T
    S = np.eye(naux) + 0.02 * (lambda B: B + B.T)(rng.standard_normal((naux, naux)))
    M = bo.TCMatrix_gwbse.Initialize(naux, 0, nmo - 1, 0, nmo - 1)
    removed = tc.fill(M, A, C, S, V)
    metric, rref = pisgw_ref(S, V, 5e-7)
    R = np.einsum("mpn,pq->mqn", fill_ref(A, C, 0, nmo - 1, 0, nmo - 1), metric)
    assert removed == rref
    assert np.linalg.norm(M.data - R) <= 1e-12 * np.linalg.norm(R)
    v, c = 6, nmo - 6
    w = np.linspace(0.3, 0.9, naux)
    hqp = np.diag(np.concatenate([np.linspace(-12, -6, v), np.linspace(1, 20, c)]))
    opt = bo.BSEOperator_Options(homo=v - 1, rpamin=0, qpmin=0, vmin=0, cmax=nmo - 1)
    ctx = bo.GpuBSEContext(w, M, hqp, opt)
    X = rng.standard_normal((v * c, 3))
    Y = bo.SingletOperator_TDA(ctx).matmul(X)
    Yr = oracle.BSEProblem(R, w, hqp, v, c).matmul_ref(X, "singlet")
    assert np.linalg.norm(Y - Yr) <= 1e-11 * np.linalg.norm(Yr)
    ctx.close()


def test_fill_errors():
    from votca_gb300 import _lib
    from votca_gb300 import bse_operator as bo
    from votca_gb300 import threecenter as tc

    A, C = _ao_problem(5, 6, 4, 2)
    with pytest.raises(_lib.BSEError):  # MO window beyond the coefficients
        tc.fill_3c_mo(bo.TCMatrix_gwbse.Initialize(5, 0, 5, 0, 3), A, C)
    with pytest.raises(_lib.BSEError):  # aux count mismatch
        tc.fill_3c_mo(bo.TCMatrix_gwbse.Initialize(4, 0, 3, 0, 3), A, C)
