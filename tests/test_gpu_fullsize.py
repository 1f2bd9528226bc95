"""Size-independent properties of the product at the benchmark sizes, where the CPU
oracle is too slow to be the reference:

- v=64, c=512, Naux=2048 (dim 32768): mixed vs FP64 products; symmetry x^T H y = y^T H x;
  linearity; the diagonal against e_i^T H e_i; Singlet = Hqp + 2 Hx - Hd term by term.
- v=128, c=1024, Naux=4096 (dim 131072 per block), full BSE: the Hamiltonian product
  [[A, B], [-B, -A]] [x; y] against separate A and B products, and sampled rows of it against
  the reference loop nest's rows (the oracle builds single rows at O(dim * Naux) each).
"""
import os

import numpy as np
import pytest

import oracle

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


def _context(v, c, naux, precision, seed):
    from votca_gb300 import bse_operator as bo
    from votca_gb300.synthetic import mmn_tensor_torch, qp_energies, screening_w

    mmn = mmn_tensor_torch(seed, naux, v + c)
    opt = bo.BSEOperator_Options(homo=v - 1, rpamin=0, qpmin=0, vmin=0, cmax=v + c - 1)
    return mmn, bo.GpuBSEContext(screening_w(seed, naux), bo.TCMatrix_gwbse(mmn),
                                 np.diag(qp_energies(seed, v, c)), opt, precision=precision)


def test_medium_workload_properties():
    from votca_gb300 import bse_operator as bo

    v, c, naux = 64, 512, 2048
    mmn, f = _context(v, c, naux, bo.PRECISION_FP64, 7)
    _, m = _context(v, c, naux, bo.PRECISION_MIXED, 7)
    n = v * c
    rng = np.random.default_rng(3)
    X = rng.standard_normal((n, 4))
    S64 = bo.SingletOperator_TDA(f)
    Yf = S64.matmul(X)
    Ym = bo.SingletOperator_TDA(m).matmul(X)
    inter = Yf - bo.HqpOperator(f).matmul(X)
    assert np.linalg.norm(Ym - Yf) / np.linalg.norm(inter) < 2e-4
    # symmetry: X^T H X is symmetric (FP64 to rounding, mixed to the split accuracy)
    G = X.T @ Yf
    assert np.max(np.abs(G - G.T)) <= 1e-11 * np.max(np.abs(G))
    Gm = X.T @ Ym
    assert np.max(np.abs(Gm - Gm.T)) <= 1e-5 * np.max(np.abs(Gm))
    # linearity
    a, b = 0.7, -1.9
    Z = S64.matmul(a * X[:, :2] + b * X[:, 2:])
    assert np.linalg.norm(Z - (a * Yf[:, :2] + b * Yf[:, 2:])) <= 1e-12 * np.linalg.norm(Z)
    # diagonal vs e_i^T H e_i on sampled pairs
    D = S64.diagonal()
    idx = rng.choice(n, 16, replace=False)
    E = np.zeros((n, 16))
    E[idx, np.arange(16)] = 1.0
    HE = S64.matmul(E)
    np.testing.assert_allclose(D[idx], HE[idx, np.arange(16)], rtol=1e-12, atol=1e-14)
    # Singlet = Hqp + 2 Hx - Hd (HdOperator carries the minus sign)
    parts = bo.HqpOperator(f).matmul(X) + 2 * bo.HxOperator(f).matmul(X) + bo.HdOperator(f).matmul(X)
    assert np.linalg.norm(parts - Yf) <= 1e-12 * np.linalg.norm(Yf)
    f.close()
    m.close()


def test_large_full_bse_hamiltonian_structure():
    from votca_gb300 import bse_operator as bo
    from votca_gb300.synthetic import qp_energies, screening_w

    v, c, naux = 128, 1024, 4096
    mmn, m = _context(v, c, naux, bo.PRECISION_MIXED, 2)
    m_w, m_hqp = screening_w(2, naux), np.diag(qp_energies(2, v, c))
    n = v * c
    rng = np.random.default_rng(5)
    X = rng.standard_normal((2 * n, 3))
    A, B = bo.SingletOperator_TDA(m), bo.SingletOperator_BTDA_B(m)
    H = bo.HamiltonianOperator(A, B).matmul(X)
    x, y = X[:n], X[n:]
    Ax, Ay, Bx, By = A.matmul(x), A.matmul(y), B.matmul(x), B.matmul(y)
    top, bot = Ax + By, -Bx - Ay
    # two split-precision evaluations of the same blocks (different column groupings): they
    # agree to the split accuracy; a misplaced block or sign would be an O(1) difference
    assert np.linalg.norm(H[:n] - top) <= 2e-4 * np.linalg.norm(top)
    assert np.linalg.norm(H[n:] - bot) <= 2e-4 * np.linalg.norm(bot)
    # B is symmetric: y^T B x = x^T B y (to the split accuracy)
    assert abs(np.sum(y * Bx) - np.sum(x * By)) <= 1e-4 * np.linalg.norm(Bx) * np.linalg.norm(y)
    # sampled rows of the Hamiltonian product against the reference loop nest's rows (each row of
    # A and B built as bse_operator.cc:52-116 builds it, then [[A, B], [-B, -A]] assembled)
    oracle.set_threads(os.cpu_count() or 1)
    prob = oracle.BSEProblem(mmn, m_w, m_hqp, v, c)
    rows = np.concatenate([[0, c - 1, n - 1], rng.choice(n, 13, replace=False)])
    XY = np.asfortranarray(np.hstack([x, y]))
    ra = prob.matmul_rows(XY, rows, "singlet")
    rb = prob.matmul_rows(XY, rows, "singlet_b")
    rq = prob.matmul_rows(XY, rows, "hqp")
    k = X.shape[1]
    top = ra[:, :k] + rb[:, k:]
    bot = -rb[:, :k] - ra[:, k:]
    inter_top = top - rq[:, :k]
    inter_bot = bot + rq[:, k:]
    e_top = np.linalg.norm(H[rows] - top) / np.linalg.norm(inter_top)
    e_bot = np.linalg.norm(H[n + rows] - bot) / np.linalg.norm(inter_bot)
    print(f"full BSE rows vs loop nest: top {e_top:.2e}, bottom {e_bot:.2e} (interaction part)")
    assert e_top <= 5e-5 and e_bot <= 5e-5, (e_top, e_bot)
    m.close()
