"""Full (non-TDA) BSE on the GPU: HAM Davidson with harmonic Ritz values."""
import numpy as np
import pytest

import oracle
from oracle.davidson_oracle import DavidsonOracle, init_matrix, ham_diagonal, full_bse_ranked_guess
from tests.conftest import is_approx
from votca_gb300.synthetic import Problem

pytestmark = pytest.mark.gpu


def _symm(n, eps, rng):
    m = eps * rng.uniform(-1, 1, (n, n))
    return m + m.T


@pytest.mark.parametrize("n,update,maxspace", [(60, "max", 0), (120, "safe", 50)])
def test_davidson_hamiltonian_kat(n, update, maxspace):
    """test_davidson.cc:283-391: [[R, C], [-C, -R]], 5 roots, tolerance normal."""
    from votca_gb300.bse_operator import DenseGpuOperator, HamiltonianOperator
    from votca_gb300.davidson import DavidsonSolver

    rng = np.random.default_rng(n)
    R = init_matrix(n, 0.01)
    C = _symm(n, 0.01, rng)
    op = DenseGpuOperator(R, C)
    H = np.block([[R, C], [-C, -R]])
    ds = DavidsonSolver()
    ds.set_tolerance("normal")
    ds.set_size_update(update)
    if maxspace:
        ds.set_max_search_space(maxspace)
    ds.set_matrix_type("HAM")
    lam, vec = ds.solve(HamiltonianOperator(op, op), 5)
    assert ds.info() == "Success"
    ev, evec = np.linalg.eig(H)
    pos = np.where(ev.real > 0)[0]
    order = pos[np.argsort(ev.real[pos])][:5]
    assert is_approx(np.sort(lam), ev.real[order], 1e-6)
    ref = evec[:, order].real
    got = vec[:, np.argsort(lam)]
    assert is_approx(ref**2 / np.sum(ref**2, axis=0), got**2, 1e-3)
    # same answer as the restated reference solver
    o = DavidsonOracle()
    o.set_tolerance("normal")
    o.set_size_update(update)
    if maxspace:
        o.max_search_space = maxspace
    o.set_matrix_type("HAM")
    lam_o, _ = o.solve(lambda X: H @ X, ham_diagonal(np.diag(R)), 5)
    assert np.allclose(np.sort(lam), np.sort(lam_o), atol=1e-6)


@pytest.mark.parametrize("prec", [0, 1])
def test_full_bse_singlets_against_dense_eig(prec):
    """Singlet [[A, B], [-B, -A]] (A = Hqp + 2Hx - Hd, B = 2Hx - Hd2), ranked guess,
    lowest 6 positive roots vs the dense eigensolver of the oracle-assembled matrix."""
    from votca_gb300 import bse_operator as bo
    from votca_gb300.bse import DavidsonOptions, solve_nonhermitian_davidson

    p = Problem(v=6, c=40, naux=96, nmo=46, seed=12)
    Mmn = bo.TCMatrix_gwbse(p.mmn)
    opt = bo.BSEOperator_Options(homo=5, rpamin=0, qpmin=0, vmin=0, cmax=45)
    ctx = bo.GpuBSEContext(p.w, Mmn, p.hqp, opt, precision=prec)
    orc = oracle.BSEProblem(p.mmn, p.w, p.hqp, 6, 40)
    A, B = orc.dense("singlet"), orc.dense("singlet_b")
    H = np.block([[A, B], [-B, -A]])
    ev = np.linalg.eigvals(H).real
    ref = np.sort(ev[ev > 0])[:6]
    lam, X, Y, ds = solve_nonhermitian_davidson(bo.SingletOperator_TDA(ctx), bo.SingletOperator_BTDA_B(ctx),
                                                DavidsonOptions(davidson_tolerance=1e-7, nmax=6))
    assert ds.info() == "Success"
    assert np.max(np.abs(np.sort(lam) - ref)) < (1e-8 if prec == 0 else 1e-5)
    nrm = np.sum(X * X, axis=0) - np.sum(Y * Y, axis=0)
    assert np.allclose(nrm, 1.0, atol=1e-10)
    # oracle: restated HAM Davidson with the same guess
    o = DavidsonOracle()
    o.set_tolerance(1e-7)
    o.max_search_space = 60
    o.set_matrix_type("HAM")
    g = full_bse_ranked_guess(np.diag(A), np.diag(B), 6)
    lam_o, _ = o.solve(lambda Z: H @ Z, ham_diagonal(np.diag(A)), 6, initial_guess=g)
    assert np.max(np.abs(np.sort(lam_o) - ref)) < 1e-8
