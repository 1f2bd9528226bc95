"""Host logic of the BSE drivers (CPU): the ranked full-BSE guess
(BuildFullBSEXRankedInitialGuess, xtp/include/votca/xtp/bse_initialization.h:47-92), the
exchange prefactor (bse.cc:136-145), the Davidson option presets, the exciton weights and the
RPA input energies (RPA::UpdateRPAInputEnergies, rpa.cc:32-73; RPA_UKS, rpa_uks.cc:41-201)."""
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


def test_rpa_input_energies_kat():
    """test_rpa.cc:41-63 (rpa_calcenergies): configure(4, 0, 9), qpmin 1, isApprox 1e-4."""
    from votca_gb300.screening import update_rpa_input_energies, update_rpa_input_energies_uks

    dft = np.array([-0.5, -0.4, -0.3, -0.2, -0.2, -0.1, 0, 0.1, 0.2, 0.3])
    gw = np.array([-0.15, -0.05, 0.05, 0.15, 0.45, 0.55, 0.65])
    ref = np.array([-0.85, -0.15, -0.05, 0.05, 0.15, 0.45, 0.55, 0.65, 0.75, 0.85])
    e = update_rpa_input_energies(dft, gw, 1, 4, 0, 9)
    assert np.linalg.norm(e - ref) <= 1e-4 * min(np.linalg.norm(e), np.linalg.norm(ref))
    np.testing.assert_allclose(e, ref, rtol=0, atol=1e-15)
    ea, eb = update_rpa_input_energies_uks(dft, dft, gw, gw, 1, 4, 4, 0, 9)   # rpamin 0: same recipe
    np.testing.assert_array_equal(ea, e)
    np.testing.assert_array_equal(eb, e)


def test_rpa_input_energies_window_offsets():
    """rpamin > 0, worked by hand: the restricted form reads the RPA vector at the absolute level
    index and shifts its first qpmin entries (rpa.cc:50-73); the unrestricted form indexes it from
    rpamin (rpa_uks.cc:163-201).  Levels 0..7, rpa window 1..7, QP levels 2..5, HOMO 3."""
    from votca_gb300.screening import update_rpa_input_energies, update_rpa_input_energies_uks

    dft = 0.1 * np.arange(8)
    gw = np.array([0.25, 0.33, 0.38, 0.60])
    e = update_rpa_input_energies(dft, gw, 2, 3, 1, 7)
    np.testing.assert_allclose(e, [-0.13, 0.02, 0.33, 0.38, 0.60, 0.9, 1.0], rtol=0, atol=1e-14)
    ea, eb = update_rpa_input_energies_uks(dft, dft, gw, gw[:3], 2, 3, 2, 1, 7)
    np.testing.assert_allclose(ea, [0.05, 0.25, 0.33, 0.38, 0.60, 0.7, 0.8], rtol=0, atol=1e-14)
    # beta: QP levels 2..4, HOMO 2 -> occ correction |0.25 - 0.2|, virt max(|0.33-0.3|, |0.38-0.4|)
    # on the DFT levels 5..7
    np.testing.assert_allclose(eb, [0.05, 0.25, 0.33, 0.38, 0.53, 0.63, 0.73], rtol=0, atol=1e-14)
    with pytest.raises(ValueError):
        update_rpa_input_energies(dft, np.zeros(7), 2, 3, 1, 7)     # QP levels past rpamax
    with pytest.raises(ValueError):
        update_rpa_input_energies(dft, gw, 0, 3, 1, 7)              # qpmin below rpamin


def test_davidson_option_setters():
    """DavidsonSolver's setters (davidsonsolver.cc:101-147): preset tolerances, the correction,
    update and matrix-type names, the reference's error text for unknown names, and the option
    struct handed to bse_davidson_solve; BSE::solve_hermitian's search space of 10 * nmax
    (bse.cc:266-293)."""
    from votca_gb300.bse import DavidsonOptions, _solver
    from votca_gb300.davidson import DavidsonSolver

    ds = DavidsonSolver()
    o = ds._options()
    assert (o.iter_max, o.tolerance, o.max_search_space, o.correction, o.update, o.matrix_type) == \
        (50, 1e-4, 0, 0, 1, 0)                      # the reference's defaults
    for name, tol in (("loose", 1e-3), ("normal", 1e-4), ("strict", 1e-5), ("lapack", 1e-9)):
        ds.set_tolerance(name)
        assert ds._options().tolerance == tol
    ds.set_tolerance(3e-7)
    ds.set_correction("OLSEN")
    ds.set_size_update("max")
    ds.set_matrix_type("HAM")
    ds.set_iter_max(7)
    ds.set_max_search_space(33)
    o = ds._options()
    assert (o.iter_max, o.tolerance, o.max_search_space, o.correction, o.update, o.matrix_type) == \
        (7, 3e-7, 33, 1, 2, 1)
    for setter, bad, text in ((ds.set_tolerance, "tight", "is not a valid Davidson tolerance"),
                              (ds.set_correction, "dpr", "is not a valid Davidson correction method"),
                              (ds.set_size_update, "SAFE", "is not a valid Davidson update"),
                              (ds.set_matrix_type, "SYM", "is not a valid Davidson matrix type")):
        with pytest.raises(RuntimeError, match=text):
            setter(bad)
    s = _solver(DavidsonOptions(davidson_correction="OLSEN", davidson_tolerance="strict",
                                davidson_update="min", davidson_maxiter=12, nmax=4))._options()
    assert (s.iter_max, s.tolerance, s.max_search_space, s.correction, s.update) == (12, 1e-5, 40, 1, 0)


def test_tcmatrix_container_mirror():
    """TCMatrix_gwbse (threecenter.h:70-142, Initialize threecenter.cc:29-48): window accessors and
    slice m as the [nsize x auxsize] matrix Mmn_[m] over the (msize, auxsize, nsize) storage."""
    from votca_gb300.bse_operator import TCMatrix_gwbse

    M = TCMatrix_gwbse.Initialize(5, 2, 6, 1, 4)
    assert (M.msize(), M.nsize(), M.auxsize()) == (5, 4, 5)
    assert (M.get_mmin(), M.get_mmax(), M.get_nmin(), M.get_nmax()) == (2, 6, 1, 4)
    assert M.data.shape == (5, 5, 4) and not M.data.any()
    M[3][2, 4] = 7.0                                   # Mmn_[3](n = 2, P = 4), a view
    assert M.data[3, 4, 2] == 7.0 and M[3].shape == (4, 5)
    d = np.arange(2 * 3 * 4, dtype=np.float64).reshape(2, 3, 4)
    T = TCMatrix_gwbse(d, mmin=1, nmin=0)
    np.testing.assert_array_equal(T[1], d[1].T)
    assert (T.get_mmax(), T.get_nmax()) == (2, 3)
