"""The UKS oracle (restated BSE_OPERATOR_UKS loops) against an independent element-wise
construction of every block, against the pinned RKS oracle where the two coincide, and the
reference's structural identities (CPU)."""
import numpy as np
import pytest

import oracle
from oracle.uks_oracle import UKS_OPERATORS, UKSProblem as Oracle
from votca_gb300.synthetic import UKSProblem

RPAMIN = 0


def _oracle(p):
    return Oracle(p.mmn_alpha, p.mmn_beta, p.w, p.hqp_alpha, p.hqp_beta, p.homo_alpha, p.homo_beta,
                  RPAMIN, p.vmin, p.cmax)


def _elementwise(p, coef):
    """Dense matrix from the element formulas of bse_operator_uks.cc (M(m, n, P) = mmn[m, P, n])."""
    cqp, cx, cd, cd2 = coef
    w = p.w
    chans = []
    for homo, M, H in ((p.homo_alpha, p.mmn_alpha, p.hqp_alpha), (p.homo_beta, p.mmn_beta, p.hqp_beta)):
        v = np.arange(p.vmin, homo + 1)
        c = np.arange(homo + 1, p.cmax + 1)
        chans.append((v, c, M, H))
    blocks = [[None, None], [None, None]]
    for so, (vo, co, Mo, Ho) in enumerate(chans):
        for si, (vi, ci, Mi, _) in enumerate(chans):
            B = np.zeros((vo.size, co.size, vi.size, ci.size))
            if so == si:
                vt = vo.size
                if cqp:
                    for a in range(vo.size):
                        B[a, :, a, :] += Ho[vt:, vt:].T   # [c1, c] = Hqp(c + vt, c1 + vt)
                    for b in range(co.size):
                        B[:, b, :, b] -= Ho[:vt, :vt].T   # [v1, v] = Hqp(v, v1)
                if cx:
                    B += cx * np.einsum("apc,bpd->acbd", Mo[vo][:, :, co], Mi[vi][:, :, ci])
                if cd:
                    # -cd sum_P w M(c1, c2) M(v1, v2)
                    B -= cd * np.einsum("cpd,p,apb->acbd", Mo[co][:, :, ci], w, Mi[vo][:, :, vi])
                if cd2:
                    B -= cd2 * np.einsum("cpb,p,apd->acbd", Mo[co][:, :, vi], w, Mi[vo][:, :, ci])
            else:
                if cd:
                    # -cd sum_P w M_out(c1, v1) M_in(v2, c2)
                    B -= cd * np.einsum("cpa,p,bpd->acbd", Mo[co][:, :, vo], w, Mi[vi][:, :, ci])
                if cd2:
                    # -cd2 sum_P w M_out(c1, v2) M_in(v1, c2), v2 / c2 in the input channel's ranges
                    B -= cd2 * np.einsum("cpb,p,apd->acbd", Mo[co][:, :, vi], w, Mi[vo][:, :, ci])
            blocks[so][si] = B.reshape(vo.size * co.size, vi.size * ci.size)
    return np.block(blocks)


@pytest.fixture(scope="module", params=[(5, 3), (3, 5)], ids=["a>b", "a<b"])
def nonsym(request):
    ha, hb = request.param
    return UKSProblem(ha, hb, vmin=1, cmax=9, naux=7, nmo=12, seed=5, symmetric=False)


@pytest.mark.parametrize("op", list(UKS_OPERATORS))
def test_loops_equal_element_formulas(nonsym, op):
    o = _oracle(nonsym)
    np.testing.assert_allclose(o.dense(op), _elementwise(nonsym, UKS_OPERATORS[op]), rtol=0, atol=1e-13)


@pytest.mark.parametrize("op", list(UKS_OPERATORS))
def test_diagonal_equals_materialised_diagonal(nonsym, op):
    o = _oracle(nonsym)
    np.testing.assert_allclose(np.diag(o.dense(op)), o.diagonal(op), rtol=0, atol=1e-14)


def test_composition_and_symmetry():
    p = UKSProblem(4, 2, vmin=0, cmax=8, naux=9, nmo=11, seed=2)
    o = _oracle(p)
    qp, hx, hd, hd2 = (o.dense(k) for k in ("qp", "hx", "hd", "hd2"))
    # HdUKSOperator / Hd2UKSOperator carry the sign (they apply -Hd, -Hd2 and their cross terms)
    np.testing.assert_allclose(o.dense("tda"), qp + hx + hd, atol=1e-13)
    np.testing.assert_allclose(o.dense("btda_b"), hx + hd2, atol=1e-13)
    for m in (qp, hx, hd, hd2):  # symmetric for (m, n)-symmetric Mmn
        np.testing.assert_allclose(m, m.T, atol=1e-13)
    # exchange stays within a spin channel; the cross-spin blocks come from Hd / Hd2 only
    na = o.alpha.size
    assert np.all(hx[:na, na:] == 0) and np.all(hx[na:, :na] == 0)
    assert np.abs(hd[:na, na:]).max() > 0 and np.abs(hd2[:na, na:]).max() > 0


def test_same_spin_blocks_equal_the_restricted_oracle():
    """Each spin channel's own block is BSE_OPERATOR<cqp,cx,cd,cd2> of that channel's Mmn:
    the restated RKS loops (pinned against the reference's golden data) give it too."""
    p = UKSProblem(4, 2, vmin=0, cmax=8, naux=9, nmo=11, seed=8, symmetric=False)
    o = _oracle(p)
    na = o.alpha.size
    parts = {"hqp": "qp", "hx": "hx", "hd": "hd", "hd2": "hd2"}
    for rks, uks in parts.items():
        D = o.dense(uks)
        for homo, M, H, sl in ((p.homo_alpha, p.mmn_alpha, p.hqp_alpha, slice(0, na)),
                               (p.homo_beta, p.mmn_beta, p.hqp_beta, slice(na, None))):
            vt, ct = homo - p.vmin + 1, p.cmax - homo
            r = oracle.BSEProblem(M, p.w, H, vt, ct, voff=p.vmin, coff=homo + 1)
            np.testing.assert_allclose(D[sl, sl], r.dense(rks, ref_loop=True), rtol=0, atol=1e-13)


def test_dense_full_bse_roots():
    """The dense branch of Solve_excitons_uks_BTDA: positive real roots of [[A, B], [-B, -A]],
    |X|^2 - |Y|^2 = 1, largest |X| positive."""
    from oracle.uks_oracle import full_bse_dense_roots

    p = UKSProblem(3, 2, vmin=0, cmax=7, naux=8, nmo=8, seed=4)
    o = _oracle(p)
    A, B = o.dense("tda"), o.dense("btda_b")
    lam, X, Y = full_bse_dense_roots(A, B, 4)
    assert np.all(np.diff(lam) >= 0) and lam[0] > 0
    H = np.block([[A, B], [-B, -A]])
    for j in range(lam.size):
        v = np.concatenate([X[:, j], Y[:, j]])
        np.testing.assert_allclose(H @ v, lam[j] * v, atol=1e-10)
        assert abs(X[:, j] @ X[:, j] - Y[:, j] @ Y[:, j] - 1.0) < 1e-12
        assert X[np.argmax(np.abs(X[:, j])), j] > 0


def test_exciton_weights_uks():
    """PrintWeightsUKS arithmetic (bse_uks.cc:520-595) on hand-made vectors (host only)."""
    from votca_gb300.bse_operator_uks import BSEOperatorUKS_Options, exciton_weights_uks

    opt = BSEOperatorUKS_Options(homo_alpha=3, homo_beta=2, rpamin=0, qpmin=0, vmin=1, cmax=6)
    na, nb = 3 * 3, 2 * 4  # alpha: v 1..3, c 4..6; beta: v 1..2, c 3..6
    X = np.zeros((na + nb, 2))
    X[1 * 3 + 2, 0] = np.sqrt(0.6)        # alpha (v=1, c=2): level 2 -> level 6
    X[na + 0 * 4 + 1, 0] = np.sqrt(0.3)   # beta  (v=0, c=1): level 1 -> level 4
    X[na + 1 * 4 + 3, 0] = np.sqrt(0.1)
    X[0, 1] = 1.0
    Y = np.zeros_like(X)
    Y[0, 1] = np.sqrt(0.2)
    r = exciton_weights_uks(opt, X, min_print_weight=0.2)
    assert abs(r[0]["alpha_weight"] - 0.6) < 1e-15 and abs(r[0]["beta_weight"] - 0.4) < 1e-15
    top = r[0]["contributions"]
    assert [(t.is_alpha, t.v, t.c) for t in top] == [(True, 1, 2), (False, 0, 1)]
    assert (top[0].homo_minus, top[0].lumo_plus) == (3 - 2, 2)   # HOMO-1 -> LUMO+2 (alpha)
    assert (top[1].homo_minus, top[1].lumo_plus) == (2 - 1, 1)   # HOMO-1 -> LUMO+1 (beta)
    full = exciton_weights_uks(opt, X, Y, min_print_weight=0.5)
    assert abs(full[1]["alpha_weight"] - 0.8) < 1e-15
    assert [(t.v, t.c) for t in full[1]["contributions"]] == [(0, 0)]
    many = exciton_weights_uks(opt, np.ones((na + nb, 1)) * 0.9, min_print_weight=0.5)
    assert len(many[0]["contributions"]) == 8 and many[0]["more_above_threshold"] == na + nb - 8


def test_product_dense_full_bse_branch_matches_oracle():
    """The product's host dense branch (used up to dim 128) against the oracle's restatement on
    the same A, B: same roots, same phase and normalisation of X and Y."""
    from oracle.uks_oracle import full_bse_dense_roots
    from votca_gb300.bse_operator_uks import _dense_full_bse

    for seed in (4, 9):
        p = UKSProblem(3, 2, vmin=0, cmax=7, naux=8, nmo=8, seed=seed)
        o = _oracle(p)
        A, B = o.dense("tda"), o.dense("btda_b")
        lam, X, Y = _dense_full_bse(A, B, 5)
        lo, Xo, Yo = full_bse_dense_roots(A, B, 5)
        np.testing.assert_allclose(lam, lo, rtol=0, atol=1e-12)
        np.testing.assert_allclose(X, Xo, rtol=0, atol=1e-10)
        np.testing.assert_allclose(Y, Yo, rtol=0, atol=1e-10)
    with pytest.raises(RuntimeError):
        _dense_full_bse(np.zeros((3, 3)), np.eye(3), 2)   # eigenvalues +-i: no real root
