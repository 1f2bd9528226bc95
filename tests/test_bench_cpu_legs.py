"""The CPU legs of bench.py on a small problem (CPU): the factorised-oracle sample times the
product on a slice of the aux index and scales it by Naux and by the waves of vectors, and the
sliced problem is the same arithmetic as the full product with the other aux functions zeroed."""
import numpy as np

import bench
import oracle
from votca_gb300.synthetic import Problem


def test_factorised_sample_scaling(monkeypatch):
    monkeypatch.setattr(bench, "V", 3)
    monkeypatch.setattr(bench, "C", 7)
    monkeypatch.setattr(bench, "K", 5)
    p = Problem(v=3, c=7, naux=16, nmo=10, seed=4)
    oracle.set_threads(2)
    t_full, desc = bench.cpu_factorised_sample(p.mmn, p.w, p.hqp, nthreads=2, p_slice=4)
    assert t_full > 0.0
    assert "4/16 aux functions for 2 vectors" in desc and "3 waves of 2" in desc


def test_factorised_slice_is_partial_product():
    p = Problem(v=3, c=7, naux=16, nmo=10, seed=5)
    X = np.asfortranarray(np.random.default_rng(0).standard_normal((21, 2)))
    sliced = oracle.BSEProblem(np.ascontiguousarray(p.mmn[:, :4, :]), p.w[:4], p.hqp, 3, 7)
    zeroed = p.mmn.copy()
    zeroed[:, 4:, :] = 0.0
    full = oracle.BSEProblem(zeroed, p.w, p.hqp, 3, 7)
    np.testing.assert_allclose(sliced.matmul_fact(X), full.matmul_fact(X), rtol=1e-13, atol=1e-13)


def test_cpu_time_to_roots_counts_operator_calls():
    roots = {"singlets": {"fp64": {"iterations": 3}, "mixed": {"iterations": 3}},
             "triplets": {"fp64": {"iterations": 5}}}
    out = bench.cpu_time_to_roots(roots, {"singlets": 47.0, "triplets": None})
    rep = out["singlets"]["cpu_reference_extrapolated"]
    assert rep["operator_calls"] == 4 and rep["seconds"] == 4 * 47.0
    assert "cpu_reference_extrapolated" not in out["triplets"]          # no triplet sample
    out = bench.cpu_time_to_roots({"singlets": {"mixed": {"iterations": 2}}}, {"singlets": 1.0})
    assert "cpu_reference_extrapolated" not in out["singlets"]          # no FP64 solve


def test_cpu_baseline_legs_small(monkeypatch):
    for name, val in (("V", 3), ("C", 7), ("K", 5), ("NAUX", 16)):
        monkeypatch.setattr(bench, name, val)
    p = Problem(v=3, c=7, naux=16, nmo=10, seed=6)
    cb = bench.cpu_baseline(p.mmn, p.w, p.hqp, factorised=True, triplet=True)
    assert cb["kind"] == "port" and cb["seconds_per_matvec"] > 0 and cb["value"] > 0
    assert "not extrapolated" in cb["sample"]
    assert cb["triplet"]["seconds_per_matvec"] > 0
    assert cb["factorised_oracle"]["seconds_per_matvec"] > 0, cb["factorised_oracle"]


def test_reference_arm_times_whole_products(monkeypatch, capsys):
    """bench.py --impl reference: every timed step is one whole product of the reference loop
    nest; one JSON line with the arm's fields."""
    import argparse
    import json

    for name, val in (("V", 3), ("C", 7), ("K", 5), ("NAUX", 16), ("NMO", 10)):
        monkeypatch.setattr(bench, name, val)
    bench.reference_arm(argparse.Namespace(steps=2, warmup=1))
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["steps"] == 2 and line["value"] > 0
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["cpu_baseline"]["value"] == line["value"]
    assert "whole k=5 singlet products" in line["cpu_baseline"]["sample"]


def test_batched_and_full_bse_cpu_legs_small():
    """The C3 leg (the Davidson restatement on a sampled subset, scaled by the reference's flops;
    one after the other on all threads, and one molecule per spawned single-threaded process)
    and the C2 leg (one Hamiltonian application, sampled) finish on tiny inputs."""
    shapes = [{"v": 2, "c": 6, "naux": 8, "nmo": 16, "seed": 1},
              {"v": 3, "c": 5, "naux": 9, "nmo": 16, "seed": 2},
              {"v": 2, "c": 7, "naux": 6, "nmo": 17, "seed": 3}]
    out = bench.cpu_baseline_batched(shapes, roots=2, tol=1e-6, n_sample=2)
    assert out["unit"] == "roots/s" and out["value"] > 0 and "2 of 3 molecules" in out["sample"]
    conc = out["concurrent"]                    # spawned single-threaded processes, one per molecule
    assert "error" not in conc, conc
    assert conc["value"] > 0 and "3 of 3 molecules (evenly spaced) solved at once" in conc["sample"]
    if "sequential_value" in out:               # the concurrent figure won
        assert out["value"] == conc["value"] > out["sequential_value"]
    else:
        assert out["value"] >= conc["value"]
    p = Problem(v=3, c=7, naux=16, nmo=10, seed=7)
    t, desc = bench.cpu_baseline_full_bse(p.mmn, p.w, p.hqp, 3, 7, 2, seconds_target=0.2)
    assert t > 0 and desc.startswith("A: ") and "; B: " in desc
