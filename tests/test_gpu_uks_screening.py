"""Unrestricted screening on the GPU: RPA_UKS eps, the dense-W UKS operator and
BSE_UKS::Perturbative_DynamicalScreening, against the reference's route restated on the CPU
(eps = 1 - R_alpha - R_beta from the raw Mmn; eigenvectors rotate both raw Mmn; w = 1/lambda
for lambda > 1e-8; expectation values of the restated UKS operators)."""
import numpy as np
import pytest

from oracle.rpa_oracle import ETA
from oracle.uks_oracle import UKSProblem as Oracle
from votca_gb300.synthetic import UKSProblem

pytestmark = pytest.mark.gpu

HA, HB, VMIN, CMAX, NAUX, NMO = 4, 2, 0, 21, 28, 24
RPAMIN, RPAMAX = 0, NMO - 1


def _energies(homo, seed):
    rng = np.random.default_rng(seed)
    occ = np.sort(rng.uniform(-16, -6, homo + 1))
    vir = np.sort(rng.uniform(0.5, 22, NMO - homo - 1))
    return np.concatenate([occ, vir])


def _eps_uks(mmns, energies, homos, freq):
    """RPA_UKS::calculate_epsilon_r (rpa_uks.cc:306-358), both channels' sums, no factor 2."""
    res = np.zeros((NAUX, NAUX))
    for mmn, e, homo in zip(mmns, energies, homos):
        lumo = homo + 1
        n_unocc = RPAMAX - lumo + 1
        for m in range(lumo - RPAMIN):
            M = mmn[m][:, -n_unocc:].T
            dE = e[-n_unocc:] - e[m]
            dm, dp = freq - dE, freq + dE
            chi = dm / (dm ** 2 + ETA ** 2) - dp / (dp ** 2 + ETA ** 2)
            res += M.T @ (chi[:, None] * M)
    return np.eye(NAUX) - res


def _oracle_at(p, ea, eb, freq):
    eps = _eps_uks((p.mmn_alpha, p.mmn_beta), (ea, eb), (HA, HB), freq)
    lam, U = np.linalg.eigh(eps)
    w = np.where(lam > 1e-8, 1.0 / np.where(lam > 1e-8, lam, 1.0), 0.0)
    ra = np.einsum("mpn,pq->mqn", p.mmn_alpha, U)
    rb = np.einsum("mpn,pq->mqn", p.mmn_beta, U)
    return Oracle(ra, rb, w, p.hqp_alpha, p.hqp_beta, HA, HB, RPAMIN, VMIN, CMAX)


def _setup():
    from votca_gb300 import bse_operator as bo
    from votca_gb300 import bse_operator_uks as bu

    p = UKSProblem(HA, HB, vmin=VMIN, cmax=CMAX, naux=NAUX, nmo=NMO, seed=21)
    ea, eb = _energies(HA, 1), _energies(HB, 2)
    p.hqp_alpha = np.diag(ea[VMIN:CMAX + 1])
    p.hqp_beta = np.diag(eb[VMIN:CMAX + 1])
    mm = bu.TCMatrix_gwbse_spin(bo.TCMatrix_gwbse(p.mmn_alpha), bo.TCMatrix_gwbse(p.mmn_beta))
    opt = bu.BSEOperatorUKS_Options(HA, HB, RPAMIN, RPAMIN, VMIN, CMAX)
    return p, ea, eb, mm, opt


def test_uks_epsilon_and_screened_operator():
    from votca_gb300 import bse_operator_uks as bu
    from votca_gb300.screening import rpa_epsilon_uks, screened_context_uks

    p, ea, eb, mm, opt = _setup()
    for freq in (0.0, 3.5):
        eps = rpa_epsilon_uks(mm, ea, eb, HA, HB, RPAMIN, RPAMAX, freq)
        ref = _eps_uks((p.mmn_alpha, p.mmn_beta), (ea, eb), (HA, HB), freq)
        np.testing.assert_allclose(eps, ref, rtol=0, atol=1e-12)
    ctx = screened_context_uks(mm, p.hqp_alpha, p.hqp_beta, opt, ea, eb, RPAMAX, 0.0)
    orc = _oracle_at(p, ea, eb, 0.0)
    X = np.random.default_rng(3).standard_normal((orc.size, 4))
    for cls, name in ((bu.ExcitonUKSOperator_TDA, "tda"), (bu.ExcitonUKSOperator_BTDA_B, "btda_b"),
                      (bu.HdUKSOperator, "hd"), (bu.Hd2UKSOperator, "hd2")):
        Y, R = cls(ctx).matmul(X), orc.matmul(X, name)
        assert np.linalg.norm(Y - R) <= 1e-11 * np.linalg.norm(R), name
        np.testing.assert_allclose(cls(ctx).diagonal(), orc.diagonal(name), rtol=1e-11, atol=1e-13)
    ctx.close()


@pytest.mark.parametrize("full", [False, True], ids=["tda", "full_bse"])
def test_uks_dynamical_screening_matches_reference_route(full):
    from votca_gb300.bse import DavidsonOptions
    from votca_gb300.bse_operator_uks import solve_excitons_uks_btda, solve_excitons_uks_tda
    from votca_gb300.screening import perturbative_dynamical_screening_uks, screened_context_uks

    p, ea, eb, mm, opt = _setup()
    ctx = screened_context_uks(mm, p.hqp_alpha, p.hqp_beta, opt, ea, eb, RPAMAX, 0.0)
    dopt = DavidsonOptions(davidson_tolerance=1e-10, nmax=3)
    if full:
        lam, X, Y, _ = solve_excitons_uks_btda(ctx, dopt)
    else:
        lam, X, _ = solve_excitons_uks_tda(ctx, dopt)
        Y = None
    ctx.close()
    dyn = perturbative_dynamical_screening_uks(mm, p.hqp_alpha, p.hqp_beta, opt, ea, eb, RPAMAX, lam, X, Y,
                                               max_iter=5, tolerance=1e-9)

    def direct(o, x, y):
        d = np.einsum("ik,ik->k", x, o.matmul(x, "hd"))
        if y is not None:
            d = d + np.einsum("ik,ik->k", y, o.matmul(y, "hd"))
            d = d + 2.0 * np.einsum("ik,ik->k", y, o.matmul(x, "hd2"))
        return d

    static = direct(_oracle_at(p, ea, eb, 0.0), X, Y)
    ref = lam.copy()
    for i in range(lam.size):
        xi = X[:, i:i + 1]
        yi = None if Y is None else Y[:, i:i + 1]
        for _ in range(5):
            old = ref[i]
            ref[i] = lam[i] + static[i] - direct(_oracle_at(p, ea, eb, old), xi, yi)[0]
            if abs(ref[i] - old) < 1e-9:
                break
    np.testing.assert_allclose(dyn, ref, rtol=0, atol=1e-9)
    assert np.all(np.abs(dyn - lam) > 1e-7)  # the frequency dependence is exercised
