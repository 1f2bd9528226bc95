"""BSE::AdjustHqpSize (bse.cc:147-186): the Hqp window of the operator for every overlap of the
BSE window [vmin, cmax] with the QP range [qpmin, qpmax] (host logic, CPU)."""
import numpy as np
import pytest

from votca_gb300.bse import adjust_hqp_size


def _inputs(qpmin, qpmax, rpamin, rpamax, seed=0):
    rng = np.random.default_rng(seed)
    g = qpmax - qpmin + 1
    H = rng.standard_normal((g, g))
    H = H + H.T + np.diag(np.arange(g) * 10.0)
    e = np.arange(rpamin, rpamax + 1) * 100.0 + 0.5  # level l -> 100 l + 0.5
    return H, e


def _expected(H, e, homo, vmin, cmax, qpmin, qpmax, rpamin):
    """Element by element: level l of the BSE window takes Hqp where both levels are QP levels,
    else the RPA energy of l on the diagonal."""
    levels = list(range(vmin, cmax + 1))
    n = len(levels)
    out = np.zeros((n, n))
    for a, la in enumerate(levels):
        for b, lb in enumerate(levels):
            if qpmin <= la <= qpmax and qpmin <= lb <= qpmax:
                out[a, b] = H[la - qpmin, lb - qpmin]
            elif a == b:
                out[a, b] = e[la - rpamin]
    return out


@pytest.mark.parametrize("case", [
    dict(vmin=2, cmax=9, qpmin=1, qpmax=10),   # window inside the QP range
    dict(vmin=2, cmax=12, qpmin=1, qpmax=9),   # virtuals beyond qpmax
    dict(vmin=0, cmax=10, qpmin=2, qpmax=10),  # occupied below qpmin
    dict(vmin=0, cmax=13, qpmin=2, qpmax=9),   # both
])
@pytest.mark.parametrize("offdiag", [True, False])
def test_adjust_hqp_size(case, offdiag):
    rpamin, rpamax, homo = 0, 15, 5
    H, e = _inputs(case["qpmin"], case["qpmax"], rpamin, rpamax)
    out = adjust_hqp_size(H, e, homo, case["vmin"], case["cmax"], case["qpmin"], case["qpmax"], rpamin,
                          use_hqp_offdiag=offdiag)
    ref = _expected(H, e, homo, case["vmin"], case["cmax"], case["qpmin"], case["qpmax"], rpamin)
    if not offdiag:
        ref = np.diag(np.diag(ref))
    np.testing.assert_array_equal(out, ref)


def test_qp_range_beyond_window_is_rejected():
    H, e = _inputs(2, 12, 0, 15)
    with pytest.raises(ValueError):
        adjust_hqp_size(H, e, 5, 0, 10, 2, 12, 0)  # vmin < qpmin and qpmax > cmax
