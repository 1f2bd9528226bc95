"""The oracle pinned against the reference's own tests and golden data (CPU)."""
import os

import numpy as np
import pytest

import oracle
from oracle.davidson_oracle import DavidsonOracle, init_matrix, ham_diagonal
from tests.conftest import is_approx
from votca_gb300.synthetic import Problem

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def methane_hqp_problem():
    """test_bse_operator.cc:74-93 geometry: homo=4, vmin=0, cmax=8 -> v=5, c=4."""
    g = np.load(os.path.join(GOLD, "bse_operator_hqp.npz"))
    naux = 17
    mmn = np.zeros((17, naux, 17))  # the Hqp operator never reads Mmn
    return oracle.BSEProblem(mmn, g["epsilon_inv"], g["Hqp"], vt=5, ct=4), g["hqp_ref"]


def test_hqp_operator_matches_reference_golden():
    prob, ref = methane_hqp_problem()
    mat = prob.matmul_ref(np.eye(prob.dim), "hqp")
    assert is_approx(mat, ref, 1e-3)
    # the golden file is printed with 6 significant digits: far tighter than 1e-3
    assert np.max(np.abs(mat - ref)) < 1e-5
    assert is_approx(np.diag(mat), prob.diagonal("hqp"), 1e-3)


@pytest.fixture(scope="module")
def small():
    p = Problem(v=5, c=7, naux=11, nmo=14, seed=3)
    return oracle.BSEProblem(p.mmn, p.w, p.hqp, p.v, p.c, voff=0, coff=p.v)


@pytest.mark.parametrize("op", list(oracle.OPERATORS))
def test_diagonal_equals_materialised_diagonal(small, op):
    mat = small.matmul_ref(np.eye(small.dim), op)
    assert np.allclose(np.diag(mat), small.diagonal(op), rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("op", list(oracle.OPERATORS))
def test_reference_loop_equals_factorised(small, op):
    X = np.random.default_rng(0).standard_normal((small.dim, 6))
    a = small.matmul_ref(X, op)
    b = small.matmul_fact(X, op)
    assert np.allclose(a, b, rtol=1e-12, atol=1e-13)


@pytest.mark.parametrize("op", list(oracle.OPERATORS))
def test_row_evaluation_equals_reference_loop(op):
    """oracle_bse_matmul_rows (rows built one at a time) against the full loop nest, with
    off-diagonal Hqp and a window that starts above rpamin (voff, coff offsets)."""
    p = Problem(v=7, c=9, naux=13, nmo=20, seed=5)
    hqp = p.hqp.copy()
    rng = np.random.default_rng(1)
    off = 0.05 * rng.standard_normal(hqp.shape)
    hqp = hqp + off + off.T
    prob = oracle.BSEProblem(p.mmn, p.w, hqp[2:, 2:], vt=5, ct=9, voff=2, coff=7)
    X = rng.standard_normal((prob.dim, 3))
    full = prob.matmul_ref(X, op)
    rows = np.array([0, 44, 3, prob.dim - 1, 17, 17])
    np.testing.assert_allclose(prob.matmul_rows(X, rows, op), full[rows], rtol=1e-12, atol=1e-13)
    with pytest.raises(IndexError):
        prob.matmul_rows(X, [prob.dim], op)


def test_operator_composition(small):
    eye = np.eye(small.dim)
    hqp, hx, hd, hd2 = (small.matmul_ref(eye, o) for o in ("hqp", "hx", "hd", "hd2"))
    # HdOperator / Hd2Operator carry the sign: they apply -Hd and -Hd2
    assert np.allclose(small.matmul_ref(eye, "singlet"), hqp + 2 * hx + hd, atol=1e-13)
    assert np.allclose(small.matmul_ref(eye, "triplet"), hqp + hd, atol=1e-13)
    assert np.allclose(small.matmul_ref(eye, "singlet_b"), 2 * hx + hd2, atol=1e-13)
    for m in (hqp, hx, hd, hd2):
        assert np.allclose(m, m.T, atol=1e-13)


def test_offsets_and_extra_mos():
    """BSE window inside a larger MO range (vmin > rpamin, rpamax > cmax)."""
    p = Problem(v=6, c=5, naux=9, nmo=6 + 5 + 5, seed=9)
    mmn = p.mmn
    sub = mmn[2:2 + 4 + 5][:, :, 2:2 + 4 + 5]
    a = oracle.BSEProblem(mmn, p.w, p.hqp[2:11, 2:11], vt=4, ct=5, voff=2, coff=6)
    b = oracle.BSEProblem(sub, p.w, p.hqp[2:11, 2:11], vt=4, ct=5, voff=0, coff=4)
    X = np.random.default_rng(1).standard_normal((20, 3))
    assert np.allclose(a.matmul_ref(X), b.matmul_ref(X), atol=1e-14)
    assert np.allclose(a.diagonal(), b.diagonal(), atol=1e-14)


def test_btda_block_structure():
    """test_bseoperator_btda.cc:55-93: Hop * I == [[A, B], [-B, -A]] at 1e-9."""
    p = Problem(v=3, c=4, naux=7, seed=5)
    prob = oracle.BSEProblem(p.mmn, p.w, p.hqp, p.v, p.c)
    eye = np.eye(2 * prob.dim)
    H = prob.ham_matmul(eye)
    A = prob.dense("singlet")
    B = prob.dense("singlet_b")
    ref = np.block([[A, B], [-B, -A]])
    assert is_approx(H, ref, 1e-9)
    H2 = prob.ham_matmul(eye, use_ref_loop=False)
    assert is_approx(H2, ref, 1e-12)


def test_vc2index():
    """test_vc2index.cc: I = ctotal*(v - vmin) + (c - cmin)."""
    from votca_gb300.indexing import vc2index

    vc = vc2index(0, 10, 10)
    assert vc.I(3, 12) == 32
    assert vc.c(vc.I(3, 12)) == 12 and vc.v(vc.I(3, 12)) == 3
    j = 0
    for v2 in range(9):
        for c2 in range(10):
            assert vc.v(j) == v2 and vc.c(j) == 10 + c2
            j += 1


# ---- Davidson KATs (test_davidson.cc) ----
@pytest.mark.parametrize("n", [100, 400])
def test_davidson_full_matrix(n):
    A = init_matrix(n, 0.01)
    ds = DavidsonOracle()
    lam, _ = ds.solve(lambda X: A @ X, np.diag(A).copy(), 10)
    ref = np.load(os.path.join(GOLD, "davidson_kat.npz"))[f"evals_{n}"]
    assert ds.info == "Success"
    assert is_approx(lam, ref, 1e-6)


def test_davidson_full_matrix_fail():
    A = init_matrix(100, 0.01)
    ds = DavidsonOracle()
    ds.iter_max = 1
    lam, _ = ds.solve(lambda X: A @ X, np.diag(A).copy(), 10)
    ref = np.load(os.path.join(GOLD, "davidson_kat.npz"))["evals_100"]
    assert ds.info == "NoConvergence"
    assert not is_approx(lam, ref, 1e-6)


@pytest.mark.parametrize("n", [100, 400])
def test_davidson_matrix_free(n):
    A = init_matrix(n, 0.01)
    ds = DavidsonOracle()
    ds.set_tolerance("normal")
    ds.set_size_update("safe")
    lam, _ = ds.solve(lambda X: A @ X, np.diag(A).copy(), 10)
    assert is_approx(lam, np.linalg.eigvalsh(A)[:10], 1e-6)


def _symm_matrix(n, eps, rng):
    m = eps * rng.uniform(-1, 1, (n, n))
    return m + m.T


@pytest.mark.parametrize("n,update,maxspace", [(60, "max", 0), (120, "safe", 50)])
def test_davidson_hamiltonian(n, update, maxspace):
    """test_davidson.cc:283-391 (HAM, harmonic Ritz), seeded in place of Eigen::Random."""
    rng = np.random.default_rng(n)
    R = init_matrix(n, 0.01)
    C = _symm_matrix(n, 0.01, rng)
    H = np.block([[R, C], [-C, -R]])
    ds = DavidsonOracle()
    ds.set_tolerance("normal")
    ds.set_size_update(update)
    if maxspace:
        ds.max_search_space = maxspace
    ds.set_matrix_type("HAM")
    lam, vec = ds.solve(lambda X: H @ X, ham_diagonal(np.diag(R)), 5)
    lam = np.sort(lam)
    ev, evec = np.linalg.eig(H)
    pos = np.where(ev.real > 0)[0]
    order = pos[np.argsort(ev.real[pos])][:5]
    assert is_approx(lam, ev.real[order], 1e-6)
    ref_vec = evec[:, order].real
    assert is_approx(ref_vec**2 / np.sum(ref_vec**2, axis=0), vec[:, np.argsort(ds.eigenvalues)] ** 2, 1e-3)


def test_gramschmidt_linear_dependence_raises():
    ds = DavidsonOracle()
    V = np.zeros((20, 4))
    V[0, 0] = V[1, 1] = V[2, 2] = V[2, 3] = 1.0  # two identical new columns
    with pytest.raises(RuntimeError, match="Linear dependencies"):
        ds.gramschmidt(V, 2)
