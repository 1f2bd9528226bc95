"""Batched solves of independent molecules (bse_davidson_solve_batch).

Molecules of uneven shape are solved (a) concurrently, each handle on its own
stream, and (b) in lockstep with one grouped launch per step.  Every
molecule's roots must equal those of its own single solve and, in FP64, the
dense eigenvalues of its TDA singlet Hamiltonian.
"""
import numpy as np
import pytest

from votca_gb300.synthetic import Problem

pytestmark = pytest.mark.gpu

SHAPES = [  # v, c, naux, seed: uneven, as in a batch of different molecules
    (4, 32, 64, 1), (5, 40, 96, 2), (7, 33, 80, 3), (4, 64, 128, 4), (6, 48, 72, 5),
    (8, 37, 100, 6), (3, 50, 64, 7), (9, 35, 120, 8), (4, 45, 90, 9), (6, 60, 110, 10),
]


def _contexts(precision):
    from votca_gb300 import bse_operator as bo

    out = []
    for v, c, naux, seed in SHAPES:
        p = Problem(v=v, c=c, naux=naux, nmo=v + c + 8, seed=seed)
        opt = bo.BSEOperator_Options(homo=v - 1, rpamin=0, qpmin=0, vmin=0, cmax=v + c - 1)
        out.append((p, bo.GpuBSEContext(p.w, bo.TCMatrix_gwbse(p.mmn), p.hqp[:v + c, :v + c], opt,
                                        precision=precision)))
    return out


def _solver(max_space=50):
    from votca_gb300.davidson import DavidsonSolver

    ds = DavidsonSolver()
    ds.set_tolerance(1e-7)
    ds.set_max_search_space(max_space)
    return ds


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_equals_single_solves(precision):
    from votca_gb300 import bse_operator as bo

    ctxs = _contexts(precision)
    ops = [bo.SingletOperator_TDA(ctx) for _, ctx in ctxs]
    nroots = 5
    ev, info, iters = _solver().solve_batch(ops, nroots, nthreads=4)
    assert ev.shape == (len(SHAPES), nroots)
    assert all(i == "Success" for i in info)
    for m, (op, (p, _)) in enumerate(zip(ops, ctxs)):
        ds = _solver()
        lam, _ = ds.solve(op, nroots)
        # same kernels, same deterministic reductions: the batch changes only the stream
        np.testing.assert_allclose(ev[m], lam, rtol=0, atol=1e-12)
        assert iters[m] == ds.num_iterations()
        if precision == 0:
            H = op.matmul(np.eye(op.rows()))
            exact = np.linalg.eigvalsh(0.5 * (H + H.T))[:nroots]
            np.testing.assert_allclose(ev[m], exact, rtol=0, atol=1e-9)
    for _, ctx in ctxs:
        ctx.close()


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("max_space", [50, 14])  # 14: restarts (restart 10 + update 7 > 14)
def test_lockstep_equals_single_solves(precision, max_space):
    from votca_gb300 import bse_operator as bo

    ctxs = _contexts(precision)
    ops = [bo.SingletOperator_TDA(ctx) for _, ctx in ctxs]
    nroots = 5
    ev, info, iters = _solver(max_space).solve_batch(ops, nroots, nthreads=0)
    assert all(i == "Success" for i in info)
    for m, op in enumerate(ops):
        ds = _solver(max_space)
        lam, _ = ds.solve(op, nroots)
        # the same iteration; the FP64 reduction orders of the grouped kernels differ, and
        # for split precision the lockstep solve of these small operators uses their dense
        # form (a differently rounded operator): 0.001 meV
        np.testing.assert_allclose(ev[m], lam, rtol=0, atol=1e-10 if precision == 0 else 1e-6)
        if precision == 0:
            assert abs(iters[m] - ds.num_iterations()) <= 1
        if precision == 0:
            H = op.matmul(np.eye(op.rows()))
            exact = np.linalg.eigvalsh(0.5 * (H + H.T))[:nroots]
            np.testing.assert_allclose(ev[m], exact, rtol=0, atol=1e-9)
    for _, ctx in ctxs:
        ctx.close()


def test_lockstep_dense_form_matches_factorised_products(monkeypatch):
    """Small split-precision operators run the lockstep solve through their dense form
    (H built once on the tensor cores); with the dense form disabled the factorised products
    are used.  Both agree with each other and with the FP64 dense eigenvalues."""
    from votca_gb300 import bse_operator as bo

    ctxs = _contexts(1)
    fp64 = _contexts(0)
    ops = [bo.SingletOperator_TDA(ctx) for _, ctx in ctxs]
    monkeypatch.setenv("VGB_BATCH_DENSE", "0")
    ev_f, info_f, _ = _solver().solve_batch(ops, 5, nthreads=0)
    monkeypatch.delenv("VGB_BATCH_DENSE")
    ev_d, info_d, _ = _solver().solve_batch(ops, 5, nthreads=0)
    assert all(i == "Success" for i in info_f + info_d)
    np.testing.assert_allclose(ev_d, ev_f, rtol=0, atol=1e-6)  # two split-precision operators
    for m, (_, c64) in enumerate(fp64):
        op = bo.SingletOperator_TDA(c64)
        H = op.matmul(np.eye(op.rows()))
        exact = np.linalg.eigvalsh(0.5 * (H + H.T))[:5]
        np.testing.assert_allclose(ev_d[m], exact, rtol=0, atol=1e-6)  # 0.001 meV
        c64.close()
    for _, ctx in ctxs:
        ctx.close()


def test_lockstep_triplets_and_tight_tolerance():
    """FP64 operators (a 1e-9 residual is below the split-precision floor)."""
    from votca_gb300 import bse_operator as bo
    from votca_gb300.davidson import DavidsonSolver

    ctxs = _contexts(0)
    ops = [bo.TripletOperator_TDA(ctx) for _, ctx in ctxs]
    ds = DavidsonSolver()
    ds.set_tolerance("lapack")
    ds.set_max_search_space(40)
    ev, info, _ = ds.solve_batch(ops, 3, nthreads=0)
    assert all(i == "Success" for i in info)
    for m, op in enumerate(ops):
        d1 = DavidsonSolver()
        d1.set_tolerance("lapack")
        d1.set_max_search_space(40)
        lam, _ = d1.solve(op, 3)
        np.testing.assert_allclose(ev[m], lam, rtol=0, atol=1e-10)
    for _, ctx in ctxs:
        ctx.close()


def test_lockstep_reports_failing_molecule():
    from votca_gb300 import _lib
    from votca_gb300 import bse_operator as bo

    ctxs = _contexts(1)[:3]
    ops = [bo.SingletOperator_TDA(ctx) for _, ctx in ctxs]
    with pytest.raises(_lib.BSEError, match="molecule 0"):
        _solver().solve_batch(ops, ops[0].rows() + 1, nthreads=0)
    with pytest.raises(_lib.BSEError):
        ds = _solver()
        ds.set_correction("OLSEN")  # lockstep supports DPR only
        ds.solve_batch(ops, 3, nthreads=0)
    ev, info, _ = _solver().solve_batch(ops, 3, nthreads=0)
    assert all(i == "Success" for i in info)
    for _, ctx in ctxs:
        ctx.close()


def test_batch_repeated_is_deterministic():
    from votca_gb300 import bse_operator as bo

    ctxs = _contexts(1)
    ops = [bo.SingletOperator_TDA(ctx) for _, ctx in ctxs]
    a, _, _ = _solver().solve_batch(ops, 5, nthreads=8)
    b, _, _ = _solver().solve_batch(ops, 5, nthreads=3)
    np.testing.assert_array_equal(a, b)
    c, _, _ = _solver().solve_batch(ops, 5, nthreads=0)
    d, _, _ = _solver().solve_batch(ops, 5, nthreads=0)
    np.testing.assert_array_equal(c, d)
    for _, ctx in ctxs:
        ctx.close()


def test_batch_reports_failing_molecule():
    from votca_gb300 import _lib
    from votca_gb300 import bse_operator as bo

    ctxs = _contexts(0)[:3]
    ops = [bo.SingletOperator_TDA(ctx) for _, ctx in ctxs]
    small = ops[0].rows()
    with pytest.raises(_lib.BSEError, match="molecule 0"):
        _solver().solve_batch(ops, small + 1, nthreads=2)  # more roots than rows
    # the handles stay usable after a failed batch
    ev, info, _ = _solver().solve_batch(ops, 3, nthreads=2)
    assert all(i == "Success" for i in info)
    for _, ctx in ctxs:
        ctx.close()


def test_batch_empty():
    ev, info, iters = _solver().solve_batch([], 5)
    assert ev.shape == (0, 5) and info == [] and iters.size == 0


def test_lockstep_autotuned_launch_shapes():
    """With at least 16 operators in a dense product round the launch shape of the grouped dense
    products is chosen by timing every candidate; the report lists the candidates and the choice,
    and the roots are those of the FP64 dense eigenproblems."""
    import json

    from votca_gb300 import _lib
    from votca_gb300 import bse_operator as bo
    from bench import autotune_table

    ctxs, dense = [], []
    for i in range(20):
        v, c, naux, seed = SHAPES[i % len(SHAPES)]
        p = Problem(v=v, c=c, naux=naux, nmo=v + c + 8, seed=100 + i)
        opt = bo.BSEOperator_Options(homo=v - 1, rpamin=0, qpmin=0, vmin=0, cmax=v + c - 1)
        ctx = bo.GpuBSEContext(p.w, bo.TCMatrix_gwbse(p.mmn), p.hqp[:v + c, :v + c], opt, precision=1)
        c64 = bo.GpuBSEContext(p.w, bo.TCMatrix_gwbse(p.mmn), p.hqp[:v + c, :v + c], opt, precision=0)
        op64 = bo.SingletOperator_TDA(c64)
        H = op64.matmul(np.eye(op64.rows()))
        dense.append(np.linalg.eigvalsh(0.5 * (H + H.T))[:5])
        c64.close()
        ctxs.append(ctx)
    ops = [bo.SingletOperator_TDA(ctx) for ctx in ctxs]
    ev, info, _ = _solver().solve_batch(ops, 5, nthreads=0)
    assert all(i == "Success" for i in info)
    np.testing.assert_allclose(ev, np.array(dense), rtol=0, atol=1e-6)
    table = autotune_table()
    dense_rows = [t for t in table if t["kernel"] == "grouped dense product"]
    assert dense_rows, table
    for t in dense_rows:
        assert t["chosen"]["bk"] in (32, 64) and t["chosen"]["operators_per_launch"] in (8, 16, 32)
        assert t["chosen"]["streams"] in (1, 4)
        assert len(t["candidates_ms"]) == 12 and all(c[3] > 0 for c in t["candidates_ms"])
        chosen = [c for c in t["candidates_ms"]
                  if c[:3] == [t["chosen"]["bk"], t["chosen"]["operators_per_launch"], t["chosen"]["streams"]]]
        assert len(chosen) == 1 and chosen[0][3] <= min(c[3] for c in t["candidates_ms"])  # the fastest
    json.dumps(table)
    for ctx in ctxs:
        ctx.close()
