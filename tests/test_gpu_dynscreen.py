"""Perturbative dynamical screening (BSE::Perturbative_DynamicalScreening) on the GPU,
against a CPU restatement of the reference's route: eps(omega) from the RPA oracle,
eigenvectors rotating Mmn in place (cumulatively, as SetupDirectInteractionOperator does),
weights 1/lambda, expectation values of -Hd on the oracle's dense operator."""
import numpy as np
import pytest

import oracle
from oracle.rpa_oracle import epsilon_r, setup_screening
from votca_gb300.synthetic import Problem

pytestmark = pytest.mark.gpu

V, C, NAUX, NROOTS = 4, 24, 40, 3
HOMO, RPAMIN, RPAMAX = V - 1, 0, V + C - 1


def _problem(seed=12):
    from votca_gb300 import bse_operator as bo

    p = Problem(v=V, c=C, naux=NAUX, nmo=V + C, seed=seed)
    energies = np.diag(p.hqp).copy()  # RPA input energies of levels rpamin..rpamax
    opt = bo.BSEOperator_Options(homo=HOMO, rpamin=RPAMIN, qpmin=0, vmin=0, cmax=V + C - 1)
    return p, energies, opt


def _reference(mmn, hqp, energies, lam, X, max_iter, tol):
    """The reference's loop, with its in-place rotations of Mmn."""
    m = mmn.copy()

    def setup(freq):
        nonlocal m
        m, w = setup_screening(m, epsilon_r(m, energies, HOMO, RPAMIN, RPAMAX, freq + 0j))
        return oracle.BSEProblem(m, w, hqp, V, C).dense("hd")

    hd0 = setup(0.0)
    static = np.einsum("ik,ij,jk->k", X, hd0, X)
    dyn = lam.copy()
    for i in range(lam.size):
        for _ in range(max_iter):
            old = dyn[i]
            hd = setup(old)
            dyn[i] = lam[i] + static[i] - X[:, i] @ hd @ X[:, i]
            if abs(dyn[i] - old) < tol:
                break
    return dyn


def test_dynamical_screening_matches_reference_route():
    from votca_gb300 import bse_operator as bo
    from votca_gb300.davidson import DavidsonSolver
    from votca_gb300.screening import perturbative_dynamical_screening, screened_context

    p, energies, opt = _problem()
    Mmn = bo.TCMatrix_gwbse(p.mmn)
    ctx = screened_context(Mmn, p.hqp, opt, energies, (HOMO, RPAMIN, RPAMAX))
    ds = DavidsonSolver()
    ds.set_tolerance(1e-10)
    ds.set_max_search_space(40)
    lam, X = ds.solve(bo.SingletOperator_TDA(ctx), NROOTS)
    ctx.close()
    dyn = perturbative_dynamical_screening(Mmn, p.hqp, opt, energies, (HOMO, RPAMIN, RPAMAX), lam, X,
                                           max_iter=6, tolerance=1e-9)
    ref = _reference(p.mmn, p.hqp, energies, lam, X, 6, 1e-9)
    np.testing.assert_allclose(dyn, ref, rtol=0, atol=1e-9)
    assert np.all(np.abs(dyn - lam) > 1e-8)  # the frequency dependence is exercised
