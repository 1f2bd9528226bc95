"""The seeded synthetic inputs follow the workload definition (CPU): Mmn symmetric in (m, n)
with N(0,1) * 0.1/sqrt(Naux) * exp(-|m-n|/40) entries, QP energies sorted in U[-20,-5] and
U[0.5,30] eV, screening w = 1 - 1/lambda with lambda ~ U[1,10], dense eps SPD with that
spectrum, batched shapes in their ranges, and every generator deterministic in its seed."""
import numpy as np
import pytest

from votca_gb300 import synthetic as sy


def test_mmn_tensor_distribution_and_symmetry():
    naux, nmo = 64, 40
    M = sy.mmn_tensor(7, naux, nmo)
    assert M.shape == (nmo, naux, nmo)
    np.testing.assert_array_equal(M, M.transpose(2, 1, 0))          # M(m, n, P) = M(n, m, P)
    m = np.arange(nmo)
    decay = np.exp(-np.abs(m[:, None] - m[None, :]) / 40.0) * (0.1 / np.sqrt(naux))
    z = M / decay[:, None, :]                                         # standard normal entries
    upper = z[np.triu_indices(nmo)[0], :, np.triu_indices(nmo)[1]]
    assert abs(upper.mean()) < 0.02 and abs(upper.std() - 1.0) < 0.02
    np.testing.assert_array_equal(M, sy.mmn_tensor(7, naux, nmo))   # deterministic
    assert not np.array_equal(M, sy.mmn_tensor(8, naux, nmo))


def test_energies_and_screening():
    e = sy.qp_energies(3, 20, 200)
    occ, vir = e[:20], e[20:]
    assert np.all(np.diff(occ) >= 0) and np.all(np.diff(vir) >= 0)
    assert occ.min() >= -20 and occ.max() <= -5 and vir.min() >= 0.5 and vir.max() <= 30
    w = sy.screening_w(3, 1000)
    lam = sy.screening_eigenvalues(3, 1000)
    assert lam.min() >= 1.0 and lam.max() <= 10.0
    np.testing.assert_allclose(w, 1.0 - 1.0 / lam)
    assert 0.0 <= w.min() and w.max() <= 0.9
    eps, Q, lam = sy.dense_screening(5, 24)
    np.testing.assert_allclose(Q.T @ Q, np.eye(24), atol=1e-12)
    np.testing.assert_allclose(np.linalg.eigvalsh(eps), np.sort(lam), atol=1e-12)


def test_batched_shapes():
    sh = sy.batched_shapes(256, seed=3)
    assert len(sh) == 256
    v = np.array([s["v"] for s in sh]); c = np.array([s["c"] for s in sh])
    naux = np.array([s["naux"] for s in sh]); nmo = np.array([s["nmo"] for s in sh])
    assert v.min() >= 4 and v.max() <= 32 and c.min() >= 32 and c.max() <= 256
    assert naux.min() >= 128 and naux.max() <= 1024
    np.testing.assert_array_equal(nmo, v + c + 8)
    assert len({s["seed"] for s in sh}) == 256                          # one seed per molecule
    assert sh == sy.batched_shapes(256, seed=3)


@pytest.mark.parametrize("symmetric", [True, False])
def test_uks_problem(symmetric):
    p = sy.UKSProblem(5, 3, vmin=1, cmax=12, naux=9, nmo=15, seed=2, symmetric=symmetric)
    assert p.mmn_alpha.shape == p.mmn_beta.shape == (15, 9, 15)
    assert not np.array_equal(p.mmn_alpha, p.mmn_beta)
    sym = np.array_equal(p.mmn_alpha, p.mmn_alpha.transpose(2, 1, 0))
    assert sym == symmetric
    assert p.hqp_alpha.shape == (5 + 7, 5 + 7) and p.hqp_beta.shape == (3 + 9, 3 + 9)


def test_mmn_tensor_torch_distribution():
    """The large-size generator (torch's seeded generator; on the CPU here): the same symmetric
    layout and entry distribution as mmn_tensor."""
    naux, nmo = 96, 48
    M = sy.mmn_tensor_torch(11, naux, nmo)
    assert M.shape == (nmo, naux, nmo) and M.dtype == np.float64
    np.testing.assert_array_equal(M, M.transpose(2, 1, 0))
    m = np.arange(nmo)
    decay = np.exp(-np.abs(m[:, None] - m[None, :]) / 40.0) * (0.1 / np.sqrt(naux))
    z = M / decay[:, None, :]
    iu = np.triu_indices(nmo)
    upper = z[iu[0], :, iu[1]]
    assert abs(upper.mean()) < 0.02 and abs(upper.std() - 1.0) < 0.02
    np.testing.assert_array_equal(M, sy.mmn_tensor_torch(11, naux, nmo))
