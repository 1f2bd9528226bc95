"""The reference's golden operator matrices for methane in 3-21G (test_bse_operator.cc:37-147)
through this library's GPU path: TCMatrix_gwbse::Fill on the device (Fill3cMO from the oracle's
AO integrals, the GW-BSE metric), MultiplyRightWithAuxMatrix(rpa_op), then the staged operator
in FP64 and in split precision, against hqp_ref / hx_ref / hd_ref / hd2_ref at the reference's
isApprox 1e-3 (and the diagonals against the products, as the reference checks them)."""
import os

import numpy as np
import pytest

from oracle import gaussian_integrals as gi
from tests.conftest import is_approx
from tests.test_integrals_golden import GOLD, methane_shells

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_golden_operator_matrices(precision):
    from votca_gb300 import bse_operator as bo
    from votca_gb300 import threecenter as tc

    shells, g = methane_shells()
    S, V, A3 = gi.overlap(shells), gi.coulomb2(shells), gi.coulomb3(shells, shells)
    M = bo.TCMatrix_gwbse.Initialize(17, 0, 16, 0, 16)
    assert tc.fill(M, A3, g["MOs"], S, V) == 0          # no auxiliary function removed
    tc.multiply_right_with_aux_matrix(M, g["rpa_op"])
    h = np.load(os.path.join(GOLD, "bse_operator_hqp.npz"))
    opt = bo.BSEOperator_Options(homo=4, rpamin=0, qpmin=0, vmin=0, cmax=8)
    ctx = bo.GpuBSEContext(h["epsilon_inv"], M, h["Hqp"], opt, precision=precision)
    assert ctx.size == 20
    eye = np.eye(20)
    tol = 2e-5 if precision == 0 else 2e-4
    for cls, ref in ((bo.HqpOperator, h["hqp_ref"]), (bo.HxOperator, g["hx_ref"]),
                     (bo.HdOperator, g["hd_ref"]), (bo.Hd2Operator, g["hd2_ref"])):
        op = cls(ctx)
        mat = op.matmul(eye)
        assert is_approx(mat, ref, 1e-3), cls.__name__
        assert np.linalg.norm(mat - ref) <= tol * np.linalg.norm(ref), cls.__name__
        assert is_approx(np.diag(mat), op.diagonal(), 1e-3), cls.__name__
    ctx.close()


def test_golden_threecenter_slices():
    """TCMatrix_gwbse::Fill on the device (window m 0..5, n 0..7) against the golden slices of
    test_threecenter_gwbse.cc:36-123 (isApprox 1e-5)."""
    from votca_gb300 import bse_operator as bo
    from votca_gb300 import threecenter as tc

    shells, _ = methane_shells()
    S, V, A3 = gi.overlap(shells), gi.coulomb2(shells), gi.coulomb3(shells, shells)
    t = np.load(os.path.join(GOLD, "threecenter_gwbse.npz"))
    M = bo.TCMatrix_gwbse.Initialize(17, 0, 5, 0, 7)
    assert tc.fill(M, A3, t["MOs"], S, V) == 0
    for k in (0, 2, 4):
        assert is_approx(M[k], t["ref%db" % k], 1e-5)


def test_golden_rpa_epsilon():
    """RPA::calculate_epsilon_r on the device at 0 and at 0.5 + 0.5i against the goldens of
    test_rpa.cc:69-140 (isApprox 1e-4), from the device Fill."""
    from votca_gb300 import bse_operator as bo
    from votca_gb300 import threecenter as tc
    from votca_gb300.screening import rpa_epsilon

    shells, _ = methane_shells()
    S, V, A3 = gi.overlap(shells), gi.coulomb2(shells), gi.coulomb3(shells, shells)
    r = np.load(os.path.join(GOLD, "rpa_methane.npz"))
    M = bo.TCMatrix_gwbse.Initialize(17, 0, 16, 0, 16)
    assert tc.fill(M, A3, r["eigenvectors"], S, V) == 0
    for freq, key in ((0.0, "r_ref"), (0.5 + 0.5j, "r_complex_ref")):
        eps = rpa_epsilon(M, r["eigenvals"], 4, 0, 16, freq)
        assert is_approx(eps, r[key], 1e-4)
        assert np.linalg.norm(eps - r[key]) <= 1e-5 * np.linalg.norm(r[key])
