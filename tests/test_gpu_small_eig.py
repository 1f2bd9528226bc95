"""The device solver of the small projected eigenproblems (bse_small_sym_eig) against numpy's
eigh, on the matrix kinds the Davidson iteration produces and on the hard cases (repeated
eigenvalues, split tridiagonals, diagonal input), in one launch of mixed sizes (matrices that fit
in shared memory and matrices that work from global memory)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _solve(mats, nws, cycles=None):
    from votca_gb300 import _lib

    L = _lib.load()
    m = np.array([a.shape[0] for a in mats], dtype=np.int64)
    nw = np.array(nws, dtype=np.int64)
    T = np.concatenate([np.asfortranarray(a).ravel(order="F") for a in mats])
    ev = np.zeros(int(nw.sum()))
    U = np.zeros(int(np.sum(m * nw)))
    P = ctypes.POINTER(ctypes.c_int64)
    _lib.check(L.bse_small_sym_eig(len(mats), m.ctypes.data_as(P), nw.ctypes.data_as(P),
                                   T.ctypes.data_as(_lib.c_dp), ev.ctypes.data_as(_lib.c_dp),
                                   U.ctypes.data_as(_lib.c_dp),
                                   cycles.ctypes.data_as(P) if cycles is not None else None))
    out, ol, ou = [], 0, 0
    for mi, wi in zip(m, nw):
        out.append((ev[ol:ol + wi], U[ou:ou + mi * wi].reshape((mi, wi), order="F")))
        ol += wi
        ou += mi * wi
    return out


def _cases():
    rng = np.random.default_rng(0)
    mats, nws, names = [], [], []

    def add(a, nw, name):
        mats.append(0.5 * (a + a.T))
        nws.append(nw)
        names.append(name)

    for m in (1, 2, 3, 7, 40, 124, 165, 200, 401):
        g = rng.standard_normal((m, m))
        add(g + g.T, min(m, 40), f"random{m}")
    # the Davidson shape: sorted diagonal (Ritz values) plus a weak coupling
    m = 150
    t = np.diag(np.sort(rng.uniform(9, 30, m))) + 1e-3 * rng.standard_normal((m, m))
    add(t, 45, "davidson")
    # repeated and nearly repeated eigenvalues
    q, _ = np.linalg.qr(rng.standard_normal((60, 60)))
    ev = np.sort(np.concatenate([[1.0] * 3, [2.0] * 2, [2.0 + 1e-9], rng.uniform(3, 10, 54)]))
    add((q * ev) @ q.T, 20, "degenerate")
    add(np.diag(np.arange(30.0, 0.0, -1.0)), 10, "diagonal")
    add(5.0 * np.eye(20), 6, "identity")
    blk = np.zeros((10, 10))
    blk[:5, :5] = 2 * np.eye(5) + 0.1
    blk[5:, 5:] = 2 * np.eye(5) + 0.1
    add(blk, 10, "split")
    return mats, nws, names


def test_small_symmetric_eigenproblems_match_eigh():
    mats, nws, names = _cases()
    res = _solve(mats, nws)
    for a, nw, name, (lam, U) in zip(mats, nws, names, res):
        ref = np.linalg.eigvalsh(a)[:nw]
        scale = max(1.0, np.abs(np.linalg.eigvalsh(a)).max())
        assert np.all(np.diff(lam) >= -1e-12 * scale), name  # ascending, as SelfAdjointEigenSolver
        assert np.max(np.abs(lam - ref)) <= 1e-12 * scale, (name, np.max(np.abs(lam - ref)))
        r = np.linalg.norm(a @ U - U * lam, axis=0).max()
        assert r <= 1e-12 * scale, (name, r)
        o = np.abs(U.T @ U - np.eye(nw)).max()
        assert o <= 1e-12, (name, o)


def test_single_job_and_errors():
    from votca_gb300 import _lib

    a = np.random.default_rng(3).standard_normal((33, 33))
    a = a + a.T
    (lam, U), = _solve([a], [33])
    np.testing.assert_allclose(lam, np.linalg.eigvalsh(a), atol=1e-12 * np.abs(lam).max())
    with pytest.raises(_lib.BSEError):
        _solve([a], [34])  # more pairs than the order


def test_davidson_shaped_problem_phase_cycles():
    """A Ritz problem of the C1 solve's shape (m = 124, 40 wanted pairs): correct, and the SM
    cycles of each phase reported (printed for the record)."""
    rng = np.random.default_rng(9)
    m = 124
    t = np.diag(np.sort(rng.uniform(9, 15, m))) + 1e-3 * rng.standard_normal((m, m))
    t = 0.5 * (t + t.T)
    cyc = np.zeros(4, dtype=np.int64)
    (lam, U), = _solve([t], [40], cyc)
    np.testing.assert_allclose(lam, np.linalg.eigvalsh(t)[:40], atol=1e-12 * 15)
    print("phase cycles (tridiagonal, bisection, inverse iteration, back-transform):", cyc.tolist())
    assert np.all(cyc > 0)
