"""The reference's end-to-end BSE goldens for methane in 3-21G (xtp/src/tests/test_bse.cc:37-330)
reproduced by the oracle chain on the CPU: AO integrals (oracle/gaussian_integrals.py) ->
TCMatrix_gwbse::Fill -> RPA eps(0) from the QP energies -> eigen-rotated screening with
1/lambda (BSE::SetupDirectInteractionOperator) -> restated BSE_OPERATOR -> dense eigenpairs and
the restated DavidsonSolver with the reference test's settings, and the perturbative dynamical
screening loop (BSE::Perturbative_DynamicalScreening).  Tolerances are the reference's
(isApprox 1e-3 on energies, subspace projections 1 to 1e-5, 0.005 / 0.05 / 0.001 for the
dynamical singlet TDA / singlet full / triplet TDA energies)."""
import os

import numpy as np
import pytest

import oracle
from oracle import gaussian_integrals as gi
from oracle.rpa_oracle import epsilon_r, setup_screening
from oracle.threecenter_oracle import fill_3c_mo, pseudo_inv_sqrt_gwbse
from oracle.uks_oracle import full_bse_dense_roots
from tests.conftest import is_approx
from tests.test_integrals_golden import GOLD, methane_shells
from votca_gb300.bse import adjust_hqp_size

HOMO, VMIN, CMAX, RPAMIN, RPAMAX, QPMIN, QPMAX = 4, 0, 16, 0, 16, 0, 16
VT, CT = HOMO - VMIN + 1, CMAX - HOMO


@pytest.fixture(scope="module")
def chain():
    shells, _ = methane_shells()
    g = np.load(os.path.join(GOLD, "bse_methane.npz"))
    S, V, A3 = gi.overlap(shells), gi.coulomb2(shells), gi.coulomb3(shells, shells)
    M = fill_3c_mo(A3, g["MOs"], 0, 16, 0, 16)
    M = np.einsum("mpn,pq->mqn", M, pseudo_inv_sqrt_gwbse(S, V, 5e-7)[0])
    e_rpa = np.diag(g["Hqp"]).copy()  # orbitals.RPAInputEnergies() = Hqp.diagonal()

    def problem(freq, offdiag=True):
        Mr, w = setup_screening(M, epsilon_r(M, e_rpa, HOMO, RPAMIN, RPAMAX, freq + 0.0j))
        H = adjust_hqp_size(g["Hqp"], e_rpa, HOMO, VMIN, CMAX, QPMIN, QPMAX, RPAMIN, use_hqp_offdiag=offdiag)
        return oracle.BSEProblem(Mr, w, H, VT, CT)

    return dict(g=g, problem=problem)


def _projection_norms(ref, vecs):
    ref = ref / np.linalg.norm(ref, axis=0)
    vecs = vecs / np.linalg.norm(vecs, axis=0)
    return np.linalg.norm(ref.T @ vecs, axis=0)


@pytest.mark.parametrize("offdiag,key", [(False, "singlets_nooffdiag_tda"), (True, "singlets_tda")])
def test_tda_singlets(chain, offdiag, key):
    g = chain["g"]
    A = chain["problem"](0.0, offdiag).dense("singlet")
    lam, vec = np.linalg.eigh(0.5 * (A + A.T))
    assert is_approx(lam[:3], g[key], 1e-3)
    assert np.abs(lam[:3] - g[key]).max() < 2e-6          # 6 printed digits
    psi = "singlets_psi_nooffdiag_tda" if not offdiag else "singlets_psi_tda"
    np.testing.assert_allclose(_projection_norms(g[psi], vec[:, :3]), 1.0, atol=1e-5)


def test_tda_triplet(chain):
    g = chain["g"]
    T = chain["problem"](0.0).dense("triplet")
    lam = np.linalg.eigvalsh(0.5 * (T + T.T))
    assert is_approx(lam[:1], g["triplets_tda"], 1e-3)
    assert abs(lam[0] - g["triplets_tda"][0]) < 2e-6
    # no eigenvector check, as in the reference (test_bse.cc:314-316 disables it): the golden
    # triplet vector has a residual of 8e-3 against this operator (its Rayleigh quotient is
    # 0.025985 for the level at 0.025895), though it lies in the threefold level to 0.99993


def test_full_bse_singlets(chain):
    g = chain["g"]
    p = chain["problem"](0.0)
    lam, X, Y = full_bse_dense_roots(p.dense("singlet"), p.dense("singlet_b"), 3)
    assert is_approx(lam, g["singlets_btda"], 1e-3)
    assert np.abs(lam - g["singlets_btda"]).max() < 2e-6
    np.testing.assert_allclose(_projection_norms(g["singlets_psi_btda"], X), 1.0, atol=1e-5)
    np.testing.assert_allclose(_projection_norms(g["singlets_psi_AR_btda"], Y), 1.0, atol=1e-5)


def _davidson(A, nroots, guess=None):
    """The restated DavidsonSolver with the settings of test_bse.cc:70-81 (DPR, lapack, safe,
    50 iterations; max search space 10 * nmax as BSE::Solve_singlets sets it)."""
    from oracle.davidson_oracle import DavidsonOracle

    d = DavidsonOracle()
    d.set_tolerance("lapack")
    d.set_correction("DPR")
    d.set_size_update("safe")
    d.max_search_space = 10 * nroots
    if guess is not None:
        d.set_matrix_type("HAM")
    lam, vec = d.solve(lambda X: A @ X, np.diag(A).copy(), nroots, initial_guess=guess)
    assert d.info == "Success"
    return lam, vec


@pytest.mark.parametrize("offdiag,key,psi", [(False, "singlets_nooffdiag_tda", "singlets_psi_nooffdiag_tda"),
                                             (True, "singlets_tda", "singlets_psi_tda")])
def test_davidson_tda_singlets(chain, offdiag, key, psi):
    """The matrix-free solve of the reference test (its TDA singlet Davidson) on the oracle
    operator: the threefold lowest level converges and spans the golden subspace."""
    g = chain["g"]
    lam, vec = _davidson(chain["problem"](0.0, offdiag).dense("singlet"), 3)
    assert is_approx(lam, g[key], 1e-3)
    assert np.abs(lam - g[key]).max() < 2e-6
    np.testing.assert_allclose(_projection_norms(g[psi], vec), 1.0, atol=1e-5)


def test_davidson_triplet_and_full_bse(chain):
    from votca_gb300.bse import full_bse_ranked_guess

    g = chain["g"]
    p = chain["problem"](0.0)
    lt, _ = _davidson(p.dense("triplet"), 1)
    assert is_approx(lt, g["triplets_tda"], 1e-3) and abs(lt[0] - g["triplets_tda"][0]) < 2e-6
    A, B = p.dense("singlet"), p.dense("singlet_b")
    n = A.shape[0]
    lb, vec = _davidson(np.block([[A, B], [-B, -A]]), 3, full_bse_ranked_guess(np.diag(A), np.diag(B), 3))
    assert is_approx(lb, g["singlets_btda"], 1e-3)
    assert np.abs(lb - g["singlets_btda"]).max() < 2e-6
    np.testing.assert_allclose(_projection_norms(g["singlets_psi_btda"], vec[:n]), 1.0, atol=1e-5)
    np.testing.assert_allclose(_projection_norms(g["singlets_psi_AR_btda"], vec[n:]), 1.0, atol=1e-5)


def _dynamical(chain, lam, X, Y=None, iters=10, tol=1e-5):
    """BSE::Perturbative_DynamicalScreening (bse.cc:610-681) on the oracle operators."""

    def direct(p, x, y):
        hd, hd2 = p.dense("hd"), p.dense("hd2")  # HdOperator / Hd2Operator: -Hd, -Hd2
        d = np.einsum("ik,ij,jk->k", x, hd, x)
        if y is not None:
            d = d + np.einsum("ik,ij,jk->k", y, hd, y) + 2.0 * np.einsum("ik,ij,jk->k", y, hd2, x)
        return d

    static = direct(chain["problem"](0.0), X, Y)
    out = lam.copy()
    for i in range(lam.size):
        xi = X[:, i:i + 1]
        yi = None if Y is None else Y[:, i:i + 1]
        for _ in range(iters):
            old = out[i]
            out[i] = lam[i] + static[i] - direct(chain["problem"](old), xi, yi)[0]
            if abs(out[i] - old) < tol:
                break
    return out


def test_dynamical_screening(chain):
    g = chain["g"]
    p = chain["problem"](0.0)
    A, T = p.dense("singlet"), p.dense("triplet")
    ls, vs = np.linalg.eigh(0.5 * (A + A.T))
    dyn = _dynamical(chain, ls[:3], vs[:, :3])
    assert is_approx(dyn, g["singlets_dynamic_TDA"], 0.005)
    assert np.abs(dyn - g["singlets_dynamic_TDA"]).max() < 1e-6   # in fact to 1e-7
    lt, vt = np.linalg.eigh(0.5 * (T + T.T))
    dt = _dynamical(chain, lt[:1], vt[:, :1])
    assert is_approx(dt, g["triplets_dynamic_TDA"], 0.001)
    assert abs(dt[0] - g["triplets_dynamic_TDA"][0]) < 1e-6
    lb, Xb, Yb = full_bse_dense_roots(A, p.dense("singlet_b"), 3)
    df = _dynamical(chain, lb, Xb, Yb)
    # the reference checks this one at 5 %; the restated formula gives 0.08909 against the
    # golden 0.08716 (2.2 %): the golden's generator is not reproduced more closely than that
    assert is_approx(df, g["singlets_dynamic_full"], 0.05)
