"""Post-solve analysis (BSE::Analyze_eh_interaction): the QP, direct and exchange parts
of each excitation energy, from GPU products, against dense oracle matrices and the
identity that the parts add up to the energy of a normalised eigenpair."""
import numpy as np
import pytest

import oracle
from votca_gb300.synthetic import Problem

pytestmark = pytest.mark.gpu

V, C, NAUX = 6, 40, 96


def _setup(seed=4):
    from votca_gb300 import bse_operator as bo

    p = Problem(v=V, c=C, naux=NAUX, nmo=V + C, seed=seed)
    opt = bo.BSEOperator_Options(homo=V - 1, rpamin=0, qpmin=0, vmin=0, cmax=V + C - 1)
    ctx = bo.GpuBSEContext(p.w, bo.TCMatrix_gwbse(p.mmn), p.hqp, opt)
    return p, ctx, oracle.BSEProblem(p.mmn, p.w, p.hqp, V, C)


@pytest.mark.parametrize("spin", ["singlet", "triplet"])
def test_tda_composition(spin):
    from votca_gb300 import bse_operator as bo
    from votca_gb300.bse import analyze_eh_interaction
    from votca_gb300.davidson import DavidsonSolver

    p, ctx, orc = _setup()
    op = bo.SingletOperator_TDA(ctx) if spin == "singlet" else bo.TripletOperator_TDA(ctx)
    ds = DavidsonSolver()
    ds.set_tolerance(1e-10)
    ds.set_max_search_space(60)
    lam, X = ds.solve(op, 6)
    a = analyze_eh_interaction(ctx, X, spin=spin)
    total = a["qp_contrib"] + a["direct_contrib"] + a["exchange_contrib"]
    np.testing.assert_allclose(total, lam, rtol=0, atol=1e-9)
    # each part against the dense oracle operators
    for key, name, pref in (("qp_contrib", "hqp", 1.0), ("direct_contrib", "hd", 1.0),
                            ("exchange_contrib", "hx", 2.0 if spin == "singlet" else 0.0)):
        D = orc.dense(name)
        ref = pref * np.einsum("ik,ij,jk->k", X, D, X)
        np.testing.assert_allclose(a[key], ref, rtol=1e-11, atol=1e-12)


def test_full_bse_composition():
    from votca_gb300 import bse_operator as bo
    from votca_gb300.bse import DavidsonOptions, analyze_eh_interaction, solve_nonhermitian_davidson

    p, ctx, orc = _setup(seed=9)
    A, B = bo.SingletOperator_TDA(ctx), bo.SingletOperator_BTDA_B(ctx)
    lam, X, Y, ds = solve_nonhermitian_davidson(A, B, DavidsonOptions(davidson_tolerance=1e-9, nmax=4))
    assert ds.info() == "Success"
    a = analyze_eh_interaction(ctx, X, Y, spin="singlet")
    total = a["qp_contrib"] + a["direct_contrib"] + a["exchange_contrib"]
    np.testing.assert_allclose(total, lam, rtol=0, atol=1e-8)
    hd2, hx = orc.dense("hd2"), orc.dense("hx")
    cross_d = 2 * np.einsum("ik,ij,jk->k", Y, hd2, X)
    hd = orc.dense("hd")
    direct = np.einsum("ik,ij,jk->k", X, hd, X) + np.einsum("ik,ij,jk->k", Y, hd, Y) + cross_d
    np.testing.assert_allclose(a["direct_contrib"], direct, rtol=1e-10, atol=1e-12)
    exch = 2 * (np.einsum("ik,ij,jk->k", X, hx, X) + np.einsum("ik,ij,jk->k", Y, hx, Y)
                + 2 * np.einsum("ik,ij,jk->k", Y, hx, X))
    np.testing.assert_allclose(a["exchange_contrib"], exch, rtol=1e-10, atol=1e-12)
