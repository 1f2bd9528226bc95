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


@pytest.mark.parametrize("m,nw", [(124, 40), (28, 7)])
def test_davidson_shaped_problem_phase_cycles(m, nw):
    """Ritz problems of the C1 solve's shape (m = 124, 40 wanted pairs; vectors of the inverse
    iteration in global memory) and of a batched 5-root solve (m = 28, 7 pairs; in shared
    memory): correct, and the SM cycles of each phase reported (printed for the record)."""
    rng = np.random.default_rng(9)
    t = np.diag(np.sort(rng.uniform(9, 15, m))) + 1e-3 * rng.standard_normal((m, m))
    t = 0.5 * (t + t.T)
    cyc = np.zeros(4, dtype=np.int64)
    (lam, U), = _solve([t], [nw], cyc)
    np.testing.assert_allclose(lam, np.linalg.eigvalsh(t)[:nw], atol=1e-12 * 15)
    assert np.abs(U.T @ U - np.eye(nw)).max() <= 1e-12
    print(f"m {m} nw {nw}: phase cycles (tridiagonal, bisection, inverse iteration, back-transform):",
          cyc.tolist())
    assert np.all(cyc > 0)


def _gen_solve(T, B, nw):
    from votca_gb300 import _lib

    L = _lib.load()
    m = T.shape[0]
    ev = np.zeros(nw)
    U = np.zeros(m * nw)
    sel = ctypes.c_int64(0)
    Tf = np.asfortranarray(T).ravel(order="F")
    Bf = np.asfortranarray(B).ravel(order="F")
    _lib.check(L.bse_small_gen_eig(m, nw, Tf.ctypes.data_as(_lib.c_dp), Bf.ctypes.data_as(_lib.c_dp),
                                   ev.ctypes.data_as(_lib.c_dp), U.ctypes.data_as(_lib.c_dp), ctypes.byref(sel)))
    return ev, U.reshape((m, nw), order="F"), sel.value


def _reference_selection(w, nw):
    """getHarmonicRitz's selection (davidsonsolver.cc:261-324) on eigenvalues w: the second
    member of each conjugate pair dropped, a stable ascending sort by real part, reversed."""
    pairs = []
    for i, x in enumerate(w):
        if x.imag == 0:
            continue
        for p in pairs:
            if p[1] < 0 and abs(w[p[0]].real - x.real) < 1e-9 and abs(w[p[0]].imag + x.imag) < 1e-9:
                p[1] = i
                break
        else:
            pairs.append([i, -1])
    seconds = {p[1] for p in pairs}
    cand = [i for i in range(len(w)) if i not in seconds]
    order = sorted(cand, key=lambda i: w[i].real)[::-1]
    return order[:nw], len(cand)


@pytest.mark.parametrize("m,nw,npairs", [(50, 20, 5), (10, 9, 3), (120, 40, 0), (7, 7, 0)])
def test_harmonic_ritz_problem_matches_eig(m, nw, npairs):
    """T u = theta B u with a known spectrum (T = B X D X^-1): real eigenvalues spread over
    [-5, 5] and npairs complex pairs below them; the device selection and vectors against
    numpy's eig with the reference's selection."""
    rng = np.random.default_rng(m + nw)
    B = rng.standard_normal((m, m)) + m ** 0.5 * np.eye(m)
    X = rng.standard_normal((m, m)) + 2.0 * np.eye(m)
    D = np.diag(np.sort(rng.uniform(-5, 5, m)))
    for p in range(npairs):  # rotation blocks: a +- ib with a below every real eigenvalue
        a, b = -10.0 + p, 0.5 + 0.1 * p
        D[2 * p:2 * p + 2, 2 * p:2 * p + 2] = [[a, b], [-b, a]]
    T = B @ X @ D @ np.linalg.inv(X)
    lam, U, sel = _gen_solve(T, B, nw)
    w, vr = np.linalg.eig(np.linalg.solve(B, T))
    idx, ncand = _reference_selection(w, nw)
    assert sel == min(ncand, nw) and ncand == m - npairs
    for c, i in enumerate(idx):
        u = U[:, c]
        assert abs(np.linalg.norm(u) - 1.0) < 1e-12
        if w[i].imag == 0:
            v = vr[:, i].real / np.linalg.norm(vr[:, i].real)
            assert abs(abs(u @ v) - 1.0) < 1e-9, (c, abs(u @ v))
            assert abs(lam[c] - u @ T @ u) < 1e-9 * np.abs(T).max()
    assert np.all(U[:, sel:] == 0) and np.all(lam[sel:] == 0)


def test_harmonic_ritz_davidson_shape():
    """The HAM Davidson's projected pencil T = V^T H V, B = V^T H H V for an orthonormal V and a
    BSE-shaped H = [[A, Bc], [-Bc, -A]]: the largest theta (the smallest positive omega)."""
    rng = np.random.default_rng(21)
    k, m, nw = 150, 90, 30
    A = np.diag(np.sort(rng.uniform(0.3, 1.5, k))) + 0.01 * rng.standard_normal((k, k))
    A = 0.5 * (A + A.T)
    Bc = 0.01 * rng.standard_normal((k, k))
    Bc = 0.5 * (Bc + Bc.T)
    H = np.block([[A, Bc], [-Bc, -A]])
    V, _ = np.linalg.qr(rng.standard_normal((2 * k, m)))
    HV = H @ V
    T, B = V.T @ HV, V.T @ (H @ HV)
    lam, U, sel = _gen_solve(T, B, nw)
    w, vr = np.linalg.eig(np.linalg.solve(B, T))
    idx, _ = _reference_selection(w, nw)
    assert sel == nw
    for c, i in enumerate(idx):
        if w[i].imag != 0:
            continue
        v = vr[:, i].real / np.linalg.norm(vr[:, i].real)
        assert abs(abs(U[:, c] @ v) - 1.0) < 1e-8, (c, abs(U[:, c] @ v))
        assert abs(lam[c] - U[:, c] @ T @ U[:, c]) < 1e-10
