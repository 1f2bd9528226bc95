"""The reference's end-to-end BSE goldens for methane in 3-21G (xtp/src/tests/test_bse.cc:37-330)
through this library's GPU path: device Fill from the oracle's AO integrals, RPA eps(0) on the
device, its Cholesky inverse as the dense screening, GPU Davidson solves (TDA singlets with and
without off-diagonal Hqp, the TDA triplet, full-BSE singlets) and the perturbative dynamical
screening, at the reference's tolerances (see tests/test_bse_golden.py for the CPU chain)."""
import os

import numpy as np
import pytest

from oracle import gaussian_integrals as gi
from tests.conftest import is_approx
from tests.test_integrals_golden import GOLD, methane_shells
from votca_gb300.bse import adjust_hqp_size

pytestmark = pytest.mark.gpu

HOMO, VMIN, CMAX, RPAMIN, RPAMAX = 4, 0, 16, 0, 16


@pytest.fixture(scope="module")
def inputs():
    from votca_gb300 import bse_operator as bo
    from votca_gb300 import threecenter as tc

    shells, _ = methane_shells()
    g = np.load(os.path.join(GOLD, "bse_methane.npz"))
    S, V, A3 = gi.overlap(shells), gi.coulomb2(shells), gi.coulomb3(shells, shells)
    M = bo.TCMatrix_gwbse.Initialize(17, 0, 16, 0, 16)
    assert tc.fill(M, A3, g["MOs"], S, V) == 0
    e = np.diag(g["Hqp"]).copy()
    opt = bo.BSEOperator_Options(homo=HOMO, rpamin=RPAMIN, qpmin=0, vmin=VMIN, cmax=CMAX)
    return dict(M=M, g=g, e=e, opt=opt)


def _hqp(inp, offdiag):
    return adjust_hqp_size(inp["g"]["Hqp"], inp["e"], HOMO, VMIN, CMAX, 0, 16, RPAMIN, use_hqp_offdiag=offdiag)


def _ctx(inp, offdiag=True):
    from votca_gb300.screening import screened_context

    return screened_context(inp["M"], _hqp(inp, offdiag), inp["opt"], inp["e"], (HOMO, RPAMIN, RPAMAX), 0.0)


def _projection_norms(ref, vecs):
    ref = ref / np.linalg.norm(ref, axis=0)
    vecs = vecs / np.linalg.norm(vecs, axis=0)
    return np.linalg.norm(ref.T @ vecs, axis=0)


def _options(nmax):
    from votca_gb300.bse import DavidsonOptions

    return DavidsonOptions(davidson_correction="DPR", davidson_tolerance="lapack", davidson_update="safe",
                           davidson_maxiter=50, nmax=nmax)


@pytest.mark.parametrize("offdiag,key,psi", [(False, "singlets_nooffdiag_tda", "singlets_psi_nooffdiag_tda"),
                                             (True, "singlets_tda", "singlets_psi_tda")])
def test_tda_singlets(inputs, offdiag, key, psi):
    from votca_gb300 import bse_operator as bo
    from votca_gb300.bse import solve_hermitian

    g = inputs["g"]
    ctx = _ctx(inputs, offdiag)
    lam, X, ds = solve_hermitian(bo.SingletOperator_TDA(ctx), _options(3))
    assert ds.info() == "Success"
    assert is_approx(lam, g[key], 1e-3)
    assert np.abs(lam - g[key]).max() < 2e-6
    np.testing.assert_allclose(_projection_norms(g[psi], X), 1.0, atol=1e-5)
    ctx.close()


def test_tda_triplet_and_full_bse(inputs):
    from votca_gb300 import bse_operator as bo
    from votca_gb300.bse import solve_hermitian, solve_nonhermitian_davidson

    g = inputs["g"]
    ctx = _ctx(inputs)
    lt, _, ds = solve_hermitian(bo.TripletOperator_TDA(ctx), _options(1))
    assert ds.info() == "Success"
    assert is_approx(lt, g["triplets_tda"], 1e-3) and abs(lt[0] - g["triplets_tda"][0]) < 2e-6
    lb, X, Y, ds = solve_nonhermitian_davidson(bo.SingletOperator_TDA(ctx), bo.SingletOperator_BTDA_B(ctx),
                                               _options(3))
    assert ds.info() == "Success"
    assert is_approx(lb, g["singlets_btda"], 1e-3)
    assert np.abs(lb - g["singlets_btda"]).max() < 2e-6
    np.testing.assert_allclose(_projection_norms(g["singlets_psi_btda"], X), 1.0, atol=1e-5)
    np.testing.assert_allclose(_projection_norms(g["singlets_psi_AR_btda"], Y), 1.0, atol=1e-5)
    ctx.close()


def test_dynamical_screening(inputs):
    from votca_gb300 import bse_operator as bo
    from votca_gb300.bse import solve_hermitian
    from votca_gb300.screening import perturbative_dynamical_screening

    g = inputs["g"]
    H = _hqp(inputs, True)
    ctx = _ctx(inputs)
    lam, X, _ = solve_hermitian(bo.SingletOperator_TDA(ctx), _options(3))
    ctx.close()
    dyn = perturbative_dynamical_screening(inputs["M"], H, inputs["opt"], inputs["e"], (HOMO, RPAMIN, RPAMAX),
                                           lam, X, None, max_iter=10, tolerance=1e-5)
    assert is_approx(dyn, g["singlets_dynamic_TDA"], 0.005)
    assert np.abs(dyn - g["singlets_dynamic_TDA"]).max() < 1e-6
