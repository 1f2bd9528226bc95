"""GPU Davidson (FP64) against the reference's Davidson KATs and the oracle."""
import os

import numpy as np
import pytest

import oracle
from oracle.davidson_oracle import DavidsonOracle, init_matrix
from tests.conftest import is_approx
from votca_gb300.synthetic import Problem

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("n", [100, 400])
def test_davidson_full_matrix_kat(n):
    """test_davidson.cc:58-100 (default options: tol 1e-4, SAFE, DPR)."""
    from votca_gb300.bse_operator import DenseGpuOperator
    from votca_gb300.davidson import DavidsonSolver

    A = init_matrix(n, 0.01)
    ds = DavidsonSolver()
    lam, _ = ds.solve(DenseGpuOperator(A), 10)
    ref = np.load(os.path.join(GOLD, "davidson_kat.npz"))[f"evals_{n}"]
    assert ds.info() == "Success"
    assert is_approx(lam, ref, 1e-6)


def test_davidson_full_matrix_fail_kat():
    """test_davidson.cc:102-119: iter_max = 1 must not reach the reference values."""
    from votca_gb300.bse_operator import DenseGpuOperator
    from votca_gb300.davidson import DavidsonSolver

    A = init_matrix(100, 0.01)
    ds = DavidsonSolver()
    ds.set_iter_max(1)
    lam, _ = ds.solve(DenseGpuOperator(A), 10)
    ref = np.load(os.path.join(GOLD, "davidson_kat.npz"))["evals_100"]
    assert ds.info() == "NoConvergence"
    assert not is_approx(lam, ref, 1e-6)


@pytest.mark.parametrize("correction", ["DPR", "OLSEN"])
@pytest.mark.parametrize("update", ["min", "safe", "max"])
def test_davidson_options_match_oracle(correction, update):
    """Every correction/update option, with restarts (max search space 40), on a
    materialised BSE matrix: GPU == oracle == dense eigensolver."""
    from votca_gb300.bse_operator import DenseGpuOperator
    from votca_gb300.davidson import DavidsonSolver

    p = Problem(v=8, c=40, naux=64, nmo=48, seed=4)
    orc = oracle.BSEProblem(p.mmn, p.w, p.hqp, 8, 40)
    A = orc.dense("singlet")
    ds = DavidsonSolver()
    ds.set_tolerance("strict")
    ds.set_correction(correction)
    ds.set_size_update(update)
    ds.set_max_search_space(40)
    lam, vec = ds.solve(DenseGpuOperator(A), 8)
    o = DavidsonOracle()
    o.set_tolerance("strict")
    o.set_correction(correction)
    o.set_size_update(update)
    o.max_search_space = 40
    lam_o, _ = o.solve(lambda X: A @ X, np.diag(A).copy(), 8)
    ref = np.linalg.eigvalsh(A)[:8]
    assert ds.info() == "Success" and o.info == "Success"
    assert ds.num_iterations() == o.i_iter
    assert np.allclose(lam, ref, atol=1e-10)
    assert np.allclose(lam, lam_o, atol=1e-10)
    res = A @ vec - vec * lam
    assert np.max(np.linalg.norm(res, axis=0)) < 1e-5


@pytest.mark.parametrize("update", ["min", "safe"])
def test_davidson_restart_on_kat_matrix(update):
    from votca_gb300.bse_operator import DenseGpuOperator
    from votca_gb300.davidson import DavidsonSolver

    A = init_matrix(300, 0.01)
    ds = DavidsonSolver()
    ds.set_tolerance("strict")
    ds.set_size_update(update)
    ds.set_max_search_space(30)
    lam, _ = ds.solve(DenseGpuOperator(A), 8)
    o = DavidsonOracle()
    o.set_tolerance("strict")
    o.set_size_update(update)
    o.max_search_space = 30
    lam_o, _ = o.solve(lambda X: A @ X, np.diag(A).copy(), 8)
    assert ds.info() == o.info == "Success"
    assert np.allclose(lam, np.linalg.eigvalsh(A)[:8], atol=1e-9)
    assert np.allclose(lam, lam_o, atol=1e-10)


def test_bse_config0_singlets_and_triplets():
    """C0: v8 c64 Naux256, 10 roots at tol 1e-7; eigenpairs vs dense eigh of the
    oracle-assembled operator and vs the oracle Davidson."""
    from votca_gb300 import bse_operator as bo
    from votca_gb300.davidson import DavidsonSolver
    from tests.test_gpu_operator import gpu_ctx, oracle_prob

    p = Problem(v=8, c=64, naux=256, nmo=72, seed=0)
    ctx = gpu_ctx(p, 8, 64)
    orc = oracle_prob(p, 8, 64)
    for name, cls in (("singlet", bo.SingletOperator_TDA), ("triplet", bo.TripletOperator_TDA)):
        H = orc.dense(name)
        ev, evec = np.linalg.eigh(H)
        ds = DavidsonSolver()
        ds.set_tolerance(1e-7)
        ds.set_max_search_space(100)
        lam, vec = ds.solve(cls(ctx), 10)
        assert ds.info() == "Success"
        assert np.max(np.abs(lam - ev[:10])) < 1e-9, name
        ov = np.abs(np.sum(vec * evec[:, :10], axis=0))
        assert np.all(ov > 1 - 1e-8), name
        o = DavidsonOracle()
        o.set_tolerance(1e-7)
        o.max_search_space = 100
        lam_o, _ = o.solve(lambda X: orc.matmul_fact(X, name), orc.diagonal(name), 10)
        assert np.max(np.abs(lam - lam_o)) < 1e-9


def test_warm_start_guess_overload():
    from votca_gb300.bse_operator import DenseGpuOperator
    from votca_gb300.davidson import DavidsonSolver

    A = init_matrix(200, 0.01)
    ev, evec = np.linalg.eigh(A)
    guess = evec[:, :12] + 1e-3 * np.random.default_rng(0).standard_normal((200, 12))
    # the reference leaves column 0 of the guess as given (gramschmidt with
    # nstart = 0 never normalises it), so callers pass unit columns
    guess /= np.linalg.norm(guess, axis=0)
    ds = DavidsonSolver()
    ds.set_tolerance("strict")
    lam, _ = ds.solve(DenseGpuOperator(A), 6, guess)
    assert ds.info() == "Success"
    assert np.allclose(lam, ev[:6], atol=1e-8)
    assert ds.num_iterations() <= 5
