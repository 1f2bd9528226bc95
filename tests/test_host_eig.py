"""The library's host eigensolvers (votca_gb300/csrc/host_eig.cpp: Householder + QL for the
Ritz problem, LU + Hessenberg + Francis QR + inverse iteration for the harmonic-Ritz problem of
HAM) against numpy/scipy on the CPU, compiled from the library's source with the host compiler."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
P = ctypes.POINTER(ctypes.c_double)


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("host_eig") / "libhost_eig_shim.so")
    src = [os.path.join(ROOT, "tests", "host_eig_shim.cpp"), os.path.join(ROOT, "votca_gb300", "csrc", "host_eig.cpp")]
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I", os.path.join(ROOT, "votca_gb300", "csrc"),
                    *src, "-o", out], check=True)
    L = ctypes.CDLL(out)
    L.shim_sym_eig.argtypes = [ctypes.c_int64, P, P, P]
    L.shim_gen_eig.argtypes = [ctypes.c_int64, P, P, P, P, P]
    return L


def _p(a):
    return a.ctypes.data_as(P)


def _sym(L, A):
    n = A.shape[0]
    A = np.asfortranarray(A)
    e, V = np.zeros(n), np.zeros((n, n), order="F")
    assert L.shim_sym_eig(n, _p(A), _p(e), _p(V)) == 0
    return e, V


@pytest.mark.parametrize("n", [1, 2, 7, 50, 200])
def test_symmetric_eigenproblem(lib, n):
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n))
    A = A + A.T
    e, V = _sym(lib, A)
    ref = np.linalg.eigvalsh(A)
    scale = max(1.0, np.abs(ref).max())
    np.testing.assert_allclose(e, ref, rtol=0, atol=1e-12 * scale)
    assert np.all(np.diff(e) >= 0)                                      # ascending
    np.testing.assert_allclose(V.T @ V, np.eye(n), atol=1e-12)          # orthonormal
    np.testing.assert_allclose(A @ V, V * e, atol=1e-11 * scale)


def test_symmetric_degenerate_and_special(lib):
    Q, _ = np.linalg.qr(np.random.default_rng(3).standard_normal((30, 30)))
    lam = np.repeat([1.0, 2.0, 5.0], 10)                    # threefold-degenerate spectrum
    A = (Q * lam) @ Q.T
    e, V = _sym(lib, A)
    np.testing.assert_allclose(e, lam, atol=1e-12)
    np.testing.assert_allclose(A @ V, V * e, atol=1e-11)
    np.testing.assert_allclose(V.T @ V, np.eye(30), atol=1e-12)
    e, V = _sym(lib, np.zeros((5, 5)))                       # zero matrix
    np.testing.assert_allclose(e, 0.0)
    np.testing.assert_allclose(V.T @ V, np.eye(5), atol=1e-14)
    D = np.diag([3.0, -1.0, 2.0])                            # already diagonal
    e, V = _sym(lib, D)
    np.testing.assert_allclose(e, [-1.0, 2.0, 3.0])


@pytest.mark.parametrize("n,seed", [(1, 0), (6, 1), (25, 2), (60, 3)])
def test_generalized_eigenproblem(lib, n, seed):
    scipy_linalg = pytest.importorskip("scipy.linalg")
    rng = np.random.default_rng(seed)
    T = np.asfortranarray(rng.standard_normal((n, n)))
    B = np.asfortranarray(rng.standard_normal((n, n)) + n * np.eye(n))
    wr, wi, V = np.zeros(n), np.zeros(n), np.zeros((n, n), order="F")
    assert lib.shim_gen_eig(n, _p(T), _p(B), _p(wr), _p(wi), _p(V)) == 0
    ref = list(scipy_linalg.eig(T, B, right=False))
    tol = 1e-9 * max(1.0, max(abs(r) for r in ref))
    for z in wr + 1j * wi:  # every eigenvalue matches a distinct reference one
        j = int(np.argmin([abs(z - r) for r in ref]))
        assert abs(z - ref[j]) <= tol
        ref.pop(j)
    # eigenvectors in LAPACK's real layout: T x = lambda B x for every (pair of) column(s)
    i = 0
    while i < n:
        if wi[i] == 0.0:
            x = V[:, i]
            lam = wr[i]
            assert np.linalg.norm(T @ x - lam * (B @ x)) <= 1e-8 * np.linalg.norm(T) * np.linalg.norm(x)
            i += 1
        else:
            x = V[:, i] + 1j * V[:, i + 1]
            lam = wr[i] + 1j * wi[i]
            assert np.linalg.norm(T @ x - lam * (B @ x)) <= 1e-8 * np.linalg.norm(T) * np.linalg.norm(x)
            assert wi[i + 1] == -wi[i]
            i += 2


def test_generalized_singular_b_is_reported(lib):
    n = 4
    T = np.asfortranarray(np.eye(n))
    B = np.asfortranarray(np.zeros((n, n)))
    wr, wi, V = np.zeros(n), np.zeros(n), np.zeros((n, n), order="F")
    assert lib.shim_gen_eig(n, _p(T), _p(B), _p(wr), _p(wi), _p(V)) == 1
