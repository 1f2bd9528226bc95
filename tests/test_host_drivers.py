"""Host logic of the BSE drivers (CPU): the ranked full-BSE guess
(BuildFullBSEXRankedInitialGuess, xtp/include/votca/xtp/bse_initialization.h:47-92), the
exchange prefactor (bse.cc:136-145) and the Davidson option presets."""
import numpy as np
import pytest

from votca_gb300.bse import exchange_prefactor, full_bse_ranked_guess


def test_ranked_guess_orders_by_full_bse_estimate():
    a = np.array([3.0, 1.0, 2.0, 2.5, 5.0, 0.5, 4.0, 6.0, 7.0, 8.0])
    b = np.array([0.0, 0.5, 1.9, 0.0, 4.9, 0.6, 0.0, 0.0, 0.0, 0.0])
    # omega = sqrt(max(0, a^2 - b^2)); index 5 has |b| > a -> omega 0
    omega = np.sqrt(np.maximum(0.0, (a - b) * (a + b)))
    g = full_bse_ranked_guess(a, b, 1)
    n = a.size
    assert g.shape == (2 * n, min(n, max(4, 8)))
    order = [int(np.argmax(g[:, k])) for k in range(g.shape[1])]
    assert order == sorted(range(n), key=lambda i: (omega[i], a[i]))[:g.shape[1]]
    assert np.all(g[n:] == 0.0) and np.all(g.sum(axis=0) == 1.0)  # X-only unit vectors
    assert order[0] == 5


def test_ranked_guess_ties_and_sizes():
    a = np.array([2.0, 1.0, 1.0, 1.0])
    b = np.zeros(4)
    g = full_bse_ranked_guess(a, b, 3)  # nguess = min(n, max(12, 8)) = n
    assert g.shape == (8, 4)
    assert [int(np.argmax(g[:, k])) for k in range(4)] == [1, 2, 3, 0]  # ties kept in index order
    with pytest.raises(RuntimeError):
        full_bse_ranked_guess(a, b[:3], 1)


def test_exchange_prefactor():
    assert exchange_prefactor("singlet") == 2.0
    assert exchange_prefactor("triplet") == 0.0


def test_exciton_weights():
    """PrintWeights (bse.cc:378-391): pairs above print_weight in pair order, HOMO-i -> LUMO+j."""
    from votca_gb300.bse import exciton_weights

    homo, vmin, cmax = 4, 1, 8          # v = 1..4, c = 5..8: 4 x 4 pairs
    X = np.zeros((16, 2))
    X[0 * 4 + 3, 0] = np.sqrt(0.3)      # v = 1, c = 8: HOMO-3 -> LUMO+3
    X[3 * 4 + 0, 0] = np.sqrt(0.7)      # v = 4, c = 5: HOMO-0 -> LUMO+0
    X[5, 1] = 1.0
    Y = np.zeros_like(X)
    Y[5, 1] = np.sqrt(0.6)              # full BSE: 1 - 0.6 = 0.4 < 0.5
    r = exciton_weights(homo, vmin, cmax, X, min_print_weight=0.25)
    assert [(a, b) for a, b, _ in r[0]] == [(3, 3), (0, 0)]       # pair order, not sorted
    assert abs(r[0][1][2] - 0.7) < 1e-15
    assert exciton_weights(homo, vmin, cmax, X, Y)[1] == []
    assert exciton_weights(homo, vmin, cmax, X)[1] == [(2, 1, 1.0)]  # v = 2, c = 6
