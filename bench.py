"""Benchmark of the BSE hot path on one GB300 (N GPUs run independent replicas).

Workload: TDA singlet BSE at v=64 occupied, c=512 virtual (dim 32768),
Naux=2048, Nmo=576, seeded synthetic inputs with the distributions of the
VOTCA-XTP GW-BSE workload definition (Mmn N(0,1)*0.1/sqrt(Naux)*exp(-|m-n|/40),
QP energies U[-20,-5] / U[0.5,30] eV, screening w = 1 - 1/lambda, lambda ~ U[1,10]).

One step = one application of the singlet operator (Hqp + 2Hx - Hd) to k=30
trial vectors (the Davidson block size at 20 roots, size_update = neigen + 10),
with X and Y resident in HBM.  value = algorithmic matvec TFLOP/s,
F = k [2 Naux vc (v+c) + 4 Naux vc + 2 vc].  The staged Mmn blocks (>5 GB)
exceed the 129 MB L2, so no L2 flush is needed between steps.

e2e: the same product through the host-pointer C ABI call (bse_op_matmul):
X copied host->device and Y device->host inside every timed step.

Also reported once, outside the timed steps: time-to-20-roots of the full
Davidson solve (tolerance 1e-7; split precision with its FP64-accurate polish
on Ozaki slice products, FP64, and slice products throughout) with the FP64
residuals of the returned roots, the C0 solve, the batched
256-molecule solve, the full-BSE solve at v=128, c=1024, Naux=4096 (32 trial
vectors per iteration, FP64 polish, an independent FP64 evaluation of its
roots), and (N = 1) the CPU figures: the reference loop nest port on one whole
product (cpu_baseline; also one whole triplet product, from which the
reference's time-to-20-roots is computed), and the factorised FP64 oracle as an
informational second figure.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64|mixed]
  python bench.py --impl reference ...   # the reference CPU path (oracle port)
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

V, C, NAUX, NMO, K, ROOTS = 64, 512, 2048, 576, 30, 20
WORKLOAD = f"tda_singlet_v{V}_c{C}_naux{NAUX}_k{K}"


def algorithmic_flops(v, c, naux, k, singlet=True):
    vc = v * c
    return k * (2.0 * naux * vc * (v + c) + (4.0 * naux * vc if singlet else 0.0) + 2.0 * vc)


def hd_stage_a_flops(v, c, naux, k):
    """c-contraction of Hd: S = Mcc X, 2 Naux v c^2 per vector."""
    return 2.0 * naux * v * c * c * k


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(x, world, device):
    """The slowest rank's time (the job's time) when N replicas run; x itself at N = 1."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(work_per_rank, seconds, world):
    """Whole-job throughput of N independent replicas (weak scaling): every rank does the
    same work, the job takes the slowest rank's time."""
    return world * work_per_rank / seconds


def make_mmn(seed, naux, nmo):
    """Seeded Mmn, layout (m, P, n) == the reference's slices laid end to end."""
    from votca_gb300.synthetic import mmn_tensor_torch

    return mmn_tensor_torch(seed, naux, nmo)


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for i, nm in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def sample_matvec(prob, v, c, k, op, seconds_target, nthreads, last_v1=False):
    """Time the reference loop nest (oracle port of bse_operator.cc:39-119 with the CPU
    branches of openmp_cuda.cc) on a bounded sample of one k-column product of `op`: a
    sub-range of c1 for the Hd/Hqp row stage and of v1 for the Hx block stage, scaled to
    the full product by the share of work sampled (the work per c1 is uniform; per v1 it
    is proportional to the number of v2 >= v1 pairs).  last_v1 samples the v1 blocks with
    the fewest pairs (large v).  Returns (seconds per product, description)."""
    X = np.asfortranarray(np.random.default_rng(1).standard_normal((v * c, k)))
    wave = min(c, nthreads)
    t0 = time.perf_counter()
    prob.matmul_ref(X, op, c1_range=(0, wave), v1_range=(0, 0))
    t_wave = time.perf_counter() - t0
    waves = int(max(1, min(c // wave, (seconds_target * 0.6) // max(t_wave, 1e-3))))
    n_c1 = wave * waves
    if waves > 1:
        t0 = time.perf_counter()
        prob.matmul_ref(X, op, c1_range=(0, n_c1), v1_range=(0, 0))
        t_rows = time.perf_counter() - t0
    else:
        t_rows = t_wave
    n_v1 = min(v, nthreads)
    v1r = (v - n_v1, v) if last_v1 else (0, n_v1)
    t0 = time.perf_counter()
    prob.matmul_ref(X, op, c1_range=(0, 0), v1_range=v1r)
    t_hx = time.perf_counter() - t0
    pairs_total = v * (v + 1) // 2
    pairs_s = sum(v - v1 for v1 in range(*v1r))
    t_full = t_rows * (c / n_c1) + t_hx * (pairs_total / pairs_s)
    desc = (f"reference loop nest (row-built Hd + v-pair Hx) on {n_c1}/{c} c1 rows and v1 blocks "
            f"{v1r[0]}..{v1r[1] - 1} ({pairs_s:.0f}/{pairs_total} pairs) of one k={k} {op} product, "
            f"extrapolated: {t_full:.1f} s per product")
    return t_full, desc


def cpu_factorised_sample(mmn, w, hqp, nthreads, p_slice=64):
    """The factorised FP64 oracle (the product summed over P in its factorised order, one
    vector per thread) on the first p_slice aux functions for one wave of min(k, threads)
    vectors, scaled to the full k-vector product: its work is linear in Naux (the Hqp part,
    2 vc (v+c) flops per vector, is not scaled and is negligible) and k vectors take
    ceil(k / threads) waves.  Returns (seconds per product, description)."""
    import oracle

    naux = mmn.shape[1]
    ps = max(1, min(p_slice, naux))
    prob = oracle.BSEProblem(np.ascontiguousarray(mmn[:, :ps, :]), w[:ps], hqp, V, C)
    kw = max(1, min(K, nthreads))
    X = np.asfortranarray(np.random.default_rng(2).standard_normal((V * C, kw)))
    t0 = time.perf_counter()
    prob.matmul_fact(X, "singlet")
    t = time.perf_counter() - t0
    waves = -(-K // kw)
    t_full = t * (naux / ps) * waves
    desc = (f"factorised FP64 oracle, one vector per thread, on {ps}/{naux} aux functions for {kw} vectors "
            f"({t:.2f} s), scaled by Naux and {waves} waves of {kw}: {t_full:.1f} s per k={K} product")
    return t_full, desc


def full_matvec(prob, v, c, k, op):
    """One whole k-column product of the reference loop nest (oracle port of
    bse_operator.cc:39-119 with the CPU branches of openmp_cuda.cc: every c1 row, every
    v1 <= v2 Hx block) on all host threads.  Returns (seconds, description)."""
    X = np.asfortranarray(np.random.default_rng(1).standard_normal((v * c, k)))
    t0 = time.perf_counter()
    prob.matmul_ref(X, op)
    t = time.perf_counter() - t0
    return t, (f"one whole k={k} {op} product of the reference loop nest (row-built Hd over all {c} c1 "
               f"rows + all {v * (v + 1) // 2} v-pair Hx blocks): {t:.1f} s, not extrapolated")


def cpu_baseline(mmn, w, hqp, factorised=False, triplet=False):
    """The reference's CPU loop nest on one whole singlet matvec at the benchmark workload
    (about 20 s on 16 cores), with all host threads; with triplet, also one whole triplet
    matvec (no Hx stage); with factorised, also the factorised FP64 oracle as an
    informational second CPU figure."""
    import oracle

    nthreads = os.cpu_count() or 1
    oracle.set_threads(nthreads)
    prob = oracle.BSEProblem(mmn, w, hqp, V, C)
    t_full, desc = full_matvec(prob, V, C, K, "singlet")
    F = algorithmic_flops(V, C, NAUX, K)
    out = {
        "value": F / t_full / 1e12, "unit": "TFLOP/s", "cores": nthreads, "kind": "port",
        "sample": desc, "seconds_per_matvec": t_full,
        "executed_tflops": ref_matvec_flops(V, C, NAUX, K) / t_full / 1e12,
    }
    if triplet:
        t_trip, desc_t = full_matvec(prob, V, C, K, "triplet")
        out["triplet"] = {"seconds_per_matvec": t_trip, "sample": desc_t}
    if factorised:
        try:
            t_fact, desc_f = cpu_factorised_sample(mmn, w, hqp, nthreads)
            out["factorised_oracle"] = {"value": F / t_fact / 1e12, "unit": "TFLOP/s", "cores": nthreads,
                                        "seconds_per_matvec": t_fact, "sample": desc_f}
        except Exception as exc:  # informational only: never costs the reference figure
            out["factorised_oracle"] = {"error": f"{type(exc).__name__}: {exc}"}
    return out


def cpu_time_to_roots(roots, per_call):
    """The reference CPU path's time-to-roots, extrapolated: the FP64 GPU solve runs the
    reference's Davidson algorithm, so the CPU solve makes as many operator calls (one per
    iteration, num_iterations() + 1), and a call of the reference loop nest costs the same for any block width up
    to the 2 (vc)^2 k term (1.5 % at k = 30), so each call is charged the sampled k = 30
    product time.  roots: the time_to_20_roots report; per_call: {"singlets": s, "triplets": s}."""
    for kind, t_call in per_call.items():
        rep = roots.get(kind, {}).get("fp64")
        if not rep or t_call is None:
            continue
        n = int(rep["iterations"]) + 1  # num_iterations() is the index of the last iteration
        roots[kind]["cpu_reference_extrapolated"] = {
            "seconds": n * t_call, "operator_calls": n, "seconds_per_call": t_call,
            "note": "operator calls of the FP64 solve x the sampled reference product time"}
    return roots


def ref_matvec_flops(v, c, naux, k):
    """Flops of the reference algorithm per TDA singlet product (rows rebuilt per call)."""
    vc = v * c
    return 2.0 * vc * vc * naux + v * (v + 1) * c * c * naux + 2.0 * vc * vc * k


def cpu_baseline_batched(shapes, roots, tol, n_sample=6, concurrent=True):
    """The reference CPU path (the DavidsonSolver restatement driving the reference
    loop nest on all host threads) on a seeded subset of the molecules, scaled to the
    whole set by the reference algorithm's flops per product; with concurrent, also one
    molecule per single-threaded process on every core, and the faster of the two is the
    figure."""
    import oracle
    from oracle.davidson_oracle import DavidsonOracle
    from votca_gb300.synthetic import qp_energies, screening_w

    nthreads = os.cpu_count() or 1
    oracle.set_threads(nthreads)
    pick = np.linspace(0, len(shapes) - 1, n_sample).round().astype(int)
    t_sample, cost_sample, iters = 0.0, 0.0, []
    for i in pick:
        sh = shapes[i]
        v, c, naux, seed = sh["v"], sh["c"], sh["naux"], sh["seed"]
        prob = oracle.BSEProblem(make_mmn(seed, naux, sh["nmo"]), screening_w(seed, naux),
                                 np.diag(qp_energies(seed, v, c)), v, c)
        d = DavidsonOracle()
        d.set_tolerance(tol)
        d.max_search_space = 10 * roots
        t0 = time.perf_counter()
        d.solve(lambda X: prob.matmul_ref(X, "singlet"), prob.diagonal("singlet"), roots)
        t_sample += time.perf_counter() - t0
        cost_sample += ref_matvec_flops(v, c, naux, 1)
        iters.append(d.i_iter)
    cost_all = sum(ref_matvec_flops(s["v"], s["c"], s["naux"], 1) for s in shapes)
    t_all = t_sample * cost_all / cost_sample
    nroots = len(shapes) * roots
    out = {
        "value": nroots / t_all, "unit": "roots/s", "cores": nthreads, "kind": "port",
        "sample": (f"{n_sample} of {len(shapes)} molecules (evenly spaced) solved one after the other "
                   f"({t_sample:.1f} s, iterations {iters}), scaled by the reference algorithm's "
                   f"flops per product to all molecules: {t_all:.0f} s"),
    }
    if concurrent:
        try:
            conc = _cpu_batched_concurrent(shapes, roots, tol, nthreads)
        except Exception as exc:  # the sequential figure stands
            conc = {"error": f"{type(exc).__name__}: {exc}"}
        out["concurrent"] = conc
        if conc.get("value", 0.0) > out["value"]:
            out["sequential_value"] = out["value"]
            out["value"] = conc["value"]
            out["cores"] = conc["cores"]
            out["sample"] = conc["sample"] + "; one after the other: " + out["sample"]
    return out


def _solve_molecule_one_thread(task):
    """Worker of the concurrent CPU leg: one molecule, one OpenMP thread (spawned process)."""
    sh, roots, tol = task
    import oracle
    from oracle.davidson_oracle import DavidsonOracle
    from votca_gb300.synthetic import mmn_tensor, qp_energies, screening_w

    oracle.set_threads(1)
    v, c, naux, seed = sh["v"], sh["c"], sh["naux"], sh["seed"]
    prob = oracle.BSEProblem(mmn_tensor(seed, naux, sh["nmo"]), screening_w(seed, naux),
                             np.diag(qp_energies(seed, v, c)), v, c)
    d = DavidsonOracle()
    d.set_tolerance(tol)
    d.max_search_space = 10 * roots
    t0 = time.perf_counter()
    d.solve(lambda X: prob.matmul_ref(X, "singlet"), prob.diagonal("singlet"), roots)
    return time.perf_counter() - t0, int(d.i_iter)


def _cpu_batched_concurrent(shapes, roots, tol, nworkers):
    """The reference run as it runs on many molecules, one molecule per process: nworkers
    spawned single-threaded processes (OpenMP and BLAS at one thread) solve as many evenly
    spaced molecules at once.  Scaled to the whole set as a queue over the workers: the busy
    seconds of the sample per worker, times the reference flops of all molecules over those of
    the sample.  The workers draw Mmn with the numpy generator (same distribution as the
    one-after-the-other leg, other values)."""
    import multiprocessing as mpr
    from concurrent.futures import ProcessPoolExecutor

    n = max(1, min(nworkers, len(shapes)))
    pick = np.linspace(0, len(shapes) - 1, n).round().astype(int)
    tasks = [(shapes[i], roots, tol) for i in pick]
    keys = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")
    saved = {k: os.environ.get(k) for k in keys}
    os.environ.update({k: "1" for k in keys})  # inherited by the spawned workers
    try:
        # an executor, not a Pool: a worker that dies raises BrokenProcessPool instead of being
        # replaced forever; every wait is bounded
        with ProcessPoolExecutor(max_workers=n, mp_context=mpr.get_context("spawn")) as ex:
            list(ex.map(abs, range(n), timeout=120))  # start the workers before the timed map
            t0 = time.perf_counter()
            res = list(ex.map(_solve_molecule_one_thread, tasks, timeout=600))
            wall = time.perf_counter() - t0
    finally:
        for k, val in saved.items():
            if val is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = val
    busy = sum(t for t, _ in res)
    cost_sample = sum(ref_matvec_flops(shapes[i]["v"], shapes[i]["c"], shapes[i]["naux"], 1) for i in pick)
    cost_all = sum(ref_matvec_flops(s["v"], s["c"], s["naux"], 1) for s in shapes)
    t_all = busy / n * cost_all / cost_sample
    return {
        "value": len(shapes) * roots / t_all, "unit": "roots/s", "cores": n, "kind": "port",
        "sample": (f"{n} of {len(shapes)} molecules (evenly spaced) solved at once, one single-threaded "
                   f"process each ({wall:.1f} s wall, {busy:.1f} busy seconds, iterations "
                   f"{[it for _, it in res]}), scaled as a queue over {n} processes by the reference "
                   f"algorithm's flops to all molecules: {t_all:.0f} s"),
    }


def cpu_baseline_full_bse(mmn, w, hqp, v, c, k, seconds_target=20.0):
    """One Hamiltonian application of the reference path at k trial vectors: A and B
    each applied to 2k columns (bseoperator_btda.h:116-149), sampled and extrapolated."""
    import oracle

    nthreads = os.cpu_count() or 1
    oracle.set_threads(nthreads)
    prob = oracle.BSEProblem(mmn, w, hqp, v, c)
    ta, da = sample_matvec(prob, v, c, 2 * k, "singlet", seconds_target / 2, nthreads, last_v1=True)
    tb, db = sample_matvec(prob, v, c, 2 * k, "singlet_b", seconds_target / 2, nthreads, last_v1=True)
    return ta + tb, f"A: {da}; B: {db} (extrapolated)"


def reference_arm(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    from votca_gb300.synthetic import qp_energies, screening_w

    import oracle

    mmn = make_mmn(1, NAUX, NMO)
    w = screening_w(1, NAUX)
    hqp = np.diag(qp_energies(1, V, C))
    nthreads = os.cpu_count() or 1
    oracle.set_threads(nthreads)
    prob = oracle.BSEProblem(mmn, w, hqp, V, C)
    X = np.asfortranarray(np.random.default_rng(1).standard_normal((V * C, K)))
    # warm-up steps: one wave of c1 rows each (caches, page faults, thread pool); not timed
    for _ in range(args.warmup):
        prob.matmul_ref(X, "singlet", c1_range=(0, min(C, nthreads)), v1_range=(0, 0))
    times = []
    for _ in range(args.steps):  # every timed step is one whole product: nothing extrapolated
        t0 = time.perf_counter()
        prob.matmul_ref(X, "singlet")
        times.append(time.perf_counter() - t0)
    t = float(np.mean(times))
    F = algorithmic_flops(V, C, NAUX, K)
    val = F / t / 1e12
    cb = {"cores": nthreads, "kind": "port",
          "sample": (f"{args.steps} whole k={K} singlet products of the reference loop nest (every c1 row, "
                     f"every v1 <= v2 Hx block), mean {t:.1f} s per product (min {min(times):.1f}, "
                     f"max {max(times):.1f}); warm-up steps: one wave of {min(C, nthreads)} c1 rows each")}
    line = {
        "impl": "reference", "metric": "bse_matvec_tflops", "value": val, "unit": "TFLOP/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "v": V, "c": C, "naux": NAUX, "nmo": NMO, "k": K},
        "cpu_baseline": {"value": val, "unit": "TFLOP/s", "cores": cb["cores"], "kind": cb["kind"],
                         "sample": cb["sample"]},
        "e2e": {"value": val, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def batched_solve(n_molecules, nthreads, roots=5, tol=1e-7, cpu=False, lockstep_only=False):
    """Independent molecules of uneven shape (v ~ U{4..32}, c ~ U{32..256},
    Naux ~ U{128..1024}, Nmo = v+c+8), lowest `roots` TDA singlets each, mixed
    precision.  Timed twice: the batched solve alone (operators staged in HBM)
    and end to end from host Mmn (upload + staging + solve + destroy)."""
    import torch

    from votca_gb300 import bse_operator as bo
    from votca_gb300.davidson import DavidsonSolver
    from votca_gb300.synthetic import batched_shapes, qp_energies, screening_w

    shapes = batched_shapes(n_molecules, seed=3)
    ctxs = []
    t_create = 0.0
    for sh in shapes:
        v, c, naux, nmo, seed = sh["v"], sh["c"], sh["naux"], sh["nmo"], sh["seed"]
        mmn = make_mmn(seed, naux, nmo)
        w = screening_w(seed, naux)
        hqp = np.diag(qp_energies(seed, v, c))
        opt = bo.BSEOperator_Options(homo=v - 1, rpamin=0, qpmin=0, vmin=0, cmax=v + c - 1)
        t0 = time.perf_counter()
        ctxs.append(bo.GpuBSEContext(w, bo.TCMatrix_gwbse(mmn), hqp, opt, precision=bo.PRECISION_MIXED))
        t_create += time.perf_counter() - t0
    ops = [bo.SingletOperator_TDA(cx) for cx in ctxs]
    ds = DavidsonSolver()
    ds.set_tolerance(tol)
    ds.set_max_search_space(10 * roots)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ev0, _, _ = ds.solve_batch(ops, roots, nthreads=0)  # first solve: per-molecule scratch allocated
    t_cold = time.perf_counter() - t0
    t0 = time.perf_counter()
    ev, info, iters = ds.solve_batch(ops, roots, nthreads=0)  # lockstep, grouped launches
    t_solve = time.perf_counter() - t0
    if lockstep_only:  # profiler workload: the cold and the warm lockstep solve only
        for cx in ctxs:
            cx.close()
        return {"workload": f"batched_tda_singlet_{n_molecules}mol_roots{roots}_lockstep",
                "first_solve_seconds": t_cold, "solve_seconds": t_solve,
                "roots_per_s": len(ops) * roots / t_solve, "iterations_mean": float(np.mean(iters))}
    # the same molecules as independent solves on host threads (one stream each); like the
    # lockstep mode, without the FP64 polish
    ds.set_fp64_polish(False)
    t0 = time.perf_counter()
    evt, _, _ = ds.solve_batch(ops, roots, nthreads=nthreads)
    t_threads = time.perf_counter() - t0
    # single-thread pass over a sample: one molecule after the other
    ns = min(32, len(ops))
    t0 = time.perf_counter()
    ev1, _, _ = ds.solve_batch(ops[:ns], roots, nthreads=1)
    t_serial = (time.perf_counter() - t0) * len(ops) / ns
    t0 = time.perf_counter()
    for cx in ctxs:
        cx.close()
    t_destroy = time.perf_counter() - t0
    nroots = len(ops) * roots
    out = {
        "workload": f"batched_tda_singlet_{n_molecules}mol_roots{roots}",
        "molecules": n_molecules, "roots_per_molecule": roots, "tolerance": tol, "precision": "mixed",
        "mode": "lockstep: one grouped launch per Davidson step over all molecules",
        "converged": int(sum(1 for x in info if x == "Success")),
        "iterations_mean": float(np.mean(iters)), "iterations_max": int(np.max(iters)),
        "solve_seconds": t_solve, "roots_per_s": nroots / t_solve,
        "solve_note": "operators staged and scratch allocated by an earlier solve of the same handles",
        "first_solve_seconds": t_cold,
        "e2e_seconds": t_create + t_cold + t_destroy,
        "e2e_roots_per_s": nroots / (t_create + t_cold + t_destroy),
        "e2e_note": "from host Mmn: upload + staging (create) + first lockstep solve + destroy",
        "repeat_identical": bool(np.array_equal(ev0, ev)),
        "threads": nthreads, "threads_roots_per_s": nroots / t_threads,
        "threads_note": "independent solves, one stream per molecule, on host threads",
        "one_thread_roots_per_s": nroots / t_serial,
        "one_thread_sample": f"first {ns} molecules, scaled",
        "lockstep_vs_threads_max_abs_diff_eV": float(np.max(np.abs(ev - evt))),
        "threads_match_one_thread": bool(np.array_equal(evt[:ns], ev1)),
        "dims": [int(s["v"] * s["c"]) for s in shapes[:4]] + ["..."],
        "autotune": autotune_table(),
        "autotune_note": "launch shapes of the grouped dense products, chosen by timing every candidate "
                         "([K box, operators per launch, streams, ms]) on the first solve's first product "
                         "round (included in first_solve_seconds)",
    }
    if cpu:
        out["cpu_baseline"] = cpu_baseline_batched(shapes, roots, tol)
    return out


def autotune_table():
    """The launch shapes the library's autotuner chose in this process (bse_autotune_report)."""
    import ctypes

    from votca_gb300 import _lib

    L = _lib.load()
    need = ctypes.c_int64(0)
    _lib.check(L.bse_autotune_report(None, 0, ctypes.byref(need)))
    buf = ctypes.create_string_buffer(max(int(need.value), 1))
    _lib.check(L.bse_autotune_report(buf, len(buf), None))
    return json.loads(buf.value.decode() or "[]")


def full_bse_report(roots=10, tol=1e-7, k=32, check=False, cpu=False):
    """Full (non-TDA) singlet BSE at v=128, c=1024 (dim 131072 per block),
    Naux=4096, Nmo=1152: HAM Davidson on [[A, B], [-B, -A]] in mixed precision,
    lowest `roots` roots; plus the HAM product throughput at k trial vectors.
    With check, the mixed eigenpairs are evaluated with FP64 products:
    omega = (X^T A X + Y^T A Y + 2 X^T B Y) / (X^T X - Y^T Y) (stationary in
    the eigenvector error) and the FP64 residual."""
    import ctypes

    import torch

    from votca_gb300 import _lib
    from votca_gb300 import bse_operator as bo
    from votca_gb300.bse import DavidsonOptions, solve_nonhermitian_davidson
    from votca_gb300.synthetic import qp_energies, screening_w

    v, c, naux, nmo, seed = 128, 1024, 4096, 1152, 2
    t0 = time.perf_counter()
    mmn = make_mmn(seed, naux, nmo)
    t_gen = time.perf_counter() - t0
    w = screening_w(seed, naux)
    hqp = np.diag(qp_energies(seed, v, c))
    opt = bo.BSEOperator_Options(homo=v - 1, rpamin=0, qpmin=0, vmin=0, cmax=v + c - 1)
    t0 = time.perf_counter()
    ctx = bo.GpuBSEContext(w, bo.TCMatrix_gwbse(mmn), hqp, opt, precision=bo.PRECISION_MIXED)
    t_stage = time.perf_counter() - t0
    A, B = bo.SingletOperator_TDA(ctx), bo.SingletOperator_BTDA_B(ctx)
    n = ctx.size
    # HAM product throughput through the host-pointer call (copies included)
    L = ctx._L
    rng = np.random.default_rng(4)
    X = np.asfortranarray(rng.standard_normal((2 * n, k)))
    Y = np.zeros_like(X)
    a = (ctypes.c_int32 * 4)(*A.coef)
    b = (ctypes.c_int32 * 4)(*B.coef)
    _lib.check(L.bse_ham_matmul(ctx.handle, a, b, bo._p(X), 2 * n, k, bo._p(Y), 2 * n))
    reps = 3
    t0 = time.perf_counter()
    for _ in range(reps):
        _lib.check(L.bse_ham_matmul(ctx.handle, a, b, bo._p(X), 2 * n, k, bo._p(Y), 2 * n))
    t_ham = (time.perf_counter() - t0) / reps
    vc = v * c
    flops_a = 2.0 * naux * vc * (v + c) + 4.0 * naux * vc + 2.0 * vc
    flops_b = 4.0 * naux * v * v * c + 4.0 * naux * vc
    F = 2 * k * (flops_a + flops_b)
    # block Davidson with k trial vectors per iteration (the configuration's 32), FP64 polish on
    dopt = DavidsonOptions(davidson_tolerance=tol, nmax=roots, davidson_block=k)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lam, Xr, Yr, ds = solve_nonhermitian_davidson(A, B, dopt)
    t_solve = time.perf_counter() - t0
    out = {
        "workload": f"full_bse_singlet_v{v}_c{c}_naux{naux}_roots{roots}", "precision": "mixed",
        "tolerance": tol, "mmn_generate_seconds": t_gen, "staging_seconds": t_stage,
        "ham_matvec": {"k": k, "seconds": t_ham, "tflops": F / t_ham / 1e12,
                       "flops": F, "note": "host-pointer call, H2D/D2H of 2 x 2n x k doubles included"},
        "time_to_roots_seconds": t_solve, "iterations": int(ds.num_iterations()), "info": ds.info(),
        "trial_vectors_per_iteration": k,
        "matvec_seconds": ds.result.seconds_matvec, "matvec_columns": int(ds.result.matvec_columns),
        "max_residual": ds.result.max_residual,
        "fp64_polish": {"applied": bool(ds.result.polished), "iterations": int(ds.result.polish_iterations),
                        "fp64_columns": int(ds.result.fp64_columns), "seconds": ds.result.seconds_polish},
        "roots_eV": [round(float(x), 9) for x in lam],
    }
    ctx.close()
    if cpu:
        t_cpu, desc = cpu_baseline_full_bse(mmn, w, hqp, v, c, k)
        out["cpu_baseline"] = {"value": F / t_cpu / 1e12, "unit": "TFLOP/s (HAM product, algorithmic)",
                               "cores": os.cpu_count() or 1, "kind": "port", "sample": desc,
                               "seconds_per_ham_product": t_cpu}
    if check:
        c64 = bo.GpuBSEContext(w, bo.TCMatrix_gwbse(mmn), hqp, opt, precision=bo.PRECISION_FP64)
        A64, B64 = bo.SingletOperator_TDA(c64), bo.SingletOperator_BTDA_B(c64)
        XY = np.asfortranarray(np.hstack([Xr, Yr]))
        AXY, BXY = A64.matmul(XY), B64.matmul(XY)
        AX, AY, BX, BY = AXY[:, :roots], AXY[:, roots:], BXY[:, :roots], BXY[:, roots:]
        num = np.sum(Xr * AX, 0) + np.sum(Yr * AY, 0) + 2 * np.sum(Xr * BY, 0)
        den = np.sum(Xr * Xr, 0) - np.sum(Yr * Yr, 0)
        om = num / den
        r1 = AX + BY - Xr * om
        r2 = -BX - AY - Yr * om
        res = np.sqrt(np.sum(r1 * r1, 0) + np.sum(r2 * r2, 0)) / np.sqrt(np.sum(Xr * Xr, 0) + np.sum(Yr * Yr, 0))
        out["fp64_check"] = {"omega_fp64_eV": [round(float(x), 9) for x in om],
                             "max_abs_diff_meV": float(np.max(np.abs(om - lam)) * 1e3),
                             "max_fp64_residual": float(res.max())}
        c64.close()
    return out


def roots_report(ctx, precision, w, Mmn, hqp, opt):
    """Time-to-20-roots (tolerance 1e-7) of singlets and triplets for each precision
    built, the per-root difference and eigenvector overlaps of mixed vs FP64, and the
    adjoint gradient of the 5 lowest singlets (FP64 eigenvectors, one call)."""
    import ctypes

    import torch

    from votca_gb300 import _lib
    from votca_gb300 import bse_operator as bo
    from votca_gb300.davidson import DavidsonSolver

    out = {}
    ctxs = {}
    for pname, pr in (("fp64", bo.PRECISION_FP64), ("mixed", bo.PRECISION_MIXED), ("sliced", bo.PRECISION_SLICED)):
        try:
            ctxs[pname] = ctx if pr == precision else bo.GpuBSEContext(w, Mmn, hqp, opt, precision=pr)
        except _lib.BSEError as e:
            out[pname] = {"unavailable": str(e)}
    for kind, cls in (("singlets", bo.SingletOperator_TDA), ("triplets", bo.TripletOperator_TDA)):
        res, vecs, lams = {}, {}, {}
        for pname, c2 in ctxs.items():
            ds = DavidsonSolver()
            ds.set_tolerance(1e-7)
            ds.set_max_search_space(10 * ROOTS)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            lam, v = ds.solve(cls(c2), ROOTS)
            dt = time.perf_counter() - t0
            vecs[pname] = v
            lams[pname] = lam
            r = ds.result
            res[pname] = {"seconds": dt, "iterations": int(ds.num_iterations()), "info": ds.info(),
                          "matvec_seconds": r.seconds_matvec, "matvec_columns": int(r.matvec_columns),
                          "max_residual": r.max_residual,
                          "roots_eV": [round(float(x), 9) for x in lam]}
            if r.polished:
                res[pname]["fp64_polish"] = {"iterations": int(r.polish_iterations),
                                             "fp64_columns": int(r.fp64_columns), "seconds": r.seconds_polish,
                                             "products": "sliced (Ozaki, tensor cores)"}
        if "fp64" in vecs and "mixed" in vecs:
            d = np.abs(np.array(res["fp64"]["roots_eV"]) - np.array(res["mixed"]["roots_eV"])) * 1e3
            res["max_abs_diff_meV"] = float(d.max())
            # |<x_fp64, x_mixed>| per root (unit vectors; 1 = identical up to sign)
            ov = np.abs(np.sum(vecs["fp64"] * vecs["mixed"], axis=0))
            res["min_eigvec_overlap"] = float(ov.min())
            res["max_one_minus_overlap"] = float((1.0 - ov).max())
            res["speedup_mixed_vs_fp64"] = res["fp64"]["seconds"] / res["mixed"]["seconds"]
            if "sliced" in vecs:
                res["speedup_sliced_vs_fp64"] = res["fp64"]["seconds"] / res["sliced"]["seconds"]
                res["sliced_max_abs_diff_meV"] = float(
                    np.max(np.abs(np.array(res["fp64"]["roots_eV"]) - np.array(res["sliced"]["roots_eV"]))) * 1e3)
            # residuals of the mixed roots under the FP64 operator (an FP64 product on the GPU)
            lam_m = lams["mixed"]
            xm = vecs["mixed"]
            A64 = cls(ctxs["fp64"])
            r64 = A64.matmul(xm) - xm * lam_m
            res["mixed"]["max_fp64_residual"] = float(np.max(np.linalg.norm(r64, axis=0)))
            # for reference: the split-precision iteration alone (no FP64 polish), its roots evaluated
            # against the FP64 operator the same way
            ds = DavidsonSolver()
            ds.set_tolerance(1e-7)
            ds.set_max_search_space(10 * ROOTS)
            ds.set_fp64_polish(False)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            lam_u, xu = ds.solve(cls(ctxs["mixed"]), ROOTS)
            dt = time.perf_counter() - t0
            ru = A64.matmul(xu) - xu * lam_u
            res["mixed_without_polish"] = {
                "seconds": dt, "iterations": int(ds.num_iterations()), "info": ds.info(),
                "max_fp64_residual": float(np.max(np.linalg.norm(ru, axis=0))),
                "max_abs_diff_meV_vs_fp64": float(np.max(np.abs(lam_u - lams["fp64"])) * 1e3),
                "note": "split-precision residuals only; not a result at the 1e-7 FP64 tolerance"}
        out[kind] = res
        if kind == "singlets" and "fp64" in ctxs:
            # adjoint: d(sum_k g_k Omega_k)/d(Mmn, Hqp, w) for the 5 lowest singlets
            c64 = ctxs["fp64"]
            X = np.asfortranarray(vecs["fp64"][:, :5])
            g = np.ones(5)
            gm = np.zeros(Mmn.data.shape)
            nh = opt.cmax - opt.vmin + 1
            gh = np.zeros((nh, nh), order="F")
            gw = np.zeros(w.shape)
            t0 = time.perf_counter()
            _lib.check(c64._L.bse_op_eig_gradient(c64.handle, 1, 2, 1, 0, bo._p(X), X.shape[0], 5, bo._p(g),
                                                  bo._p(gm), bo._p(gh), bo._p(gw)))
            out["adjoint_5_singlets"] = {
                "seconds": time.perf_counter() - t0,
                "note": "one bse_op_eig_gradient call: gradients w.r.t. all Mmn entries (5.4 GB, copied "
                        "to the host), the Hqp window and the screening; FP64"}
            # the same gradient kept on the device in block layouts (no 5.4 GB copy): FP64 handle,
            # and the split-precision handle (cc-block contractions as slice products)
            dev = {}
            for pname in ("fp64", "mixed"):
                if pname not in ctxs:
                    continue
                cc = ctxs[pname]
                Xd = torch.tensor(np.ascontiguousarray(X.T), device="cuda")  # row j = vector j
                outs = [torch.empty(n, dtype=torch.float64, device="cuda") for n in (
                    NAUX * V * C, NAUX * V * C, NAUX * V * V, NAUX * C * C, (V + C) ** 2, NAUX)]
                A4 = (ctypes.c_int32 * 4)(1, 2, 1, 0)
                B4 = (ctypes.c_int32 * 4)(0, 0, 0, 0)
                times = []
                for _ in range(2):
                    torch.cuda.synchronize()
                    t0 = time.perf_counter()
                    _lib.check(cc._L.bse_op_eig_gradient_device(
                        cc.handle, A4, B4, ctypes.c_void_p(Xd.data_ptr()), None, V * C, 5, bo._p(g),
                        *[ctypes.c_void_p(o.data_ptr()) for o in outs], ctypes.c_void_p(0)))
                    times.append(time.perf_counter() - t0)
                dev[pname] = {"seconds": times[-1], "grad_cc": outs[3]}
            if "fp64" in dev and "mixed" in dev:
                a, b = dev["fp64"]["grad_cc"], dev["mixed"]["grad_cc"]
                rel = float(torch.linalg.norm(b - a) / torch.linalg.norm(a))
            else:
                rel = None
            out["adjoint_5_singlets_device"] = {
                **{p_: {"seconds": d_["seconds"]} for p_, d_ in dev.items()},
                "mixed_vs_fp64_grad_cc_rel": rel,
                "note": "bse_op_eig_gradient_device, block gradients left on the device; the split-precision "
                        "handle forms the cc-block contractions as FP64-accurate slice products"}
    for pname, c2 in ctxs.items():
        if c2 is not ctx:
            c2.close()
    return out


def c0_report(cpu=True):
    """The reference's CPU-runnable case (v=8, c=64, Naux=256, 10 roots, tolerance 1e-7):
    full solves on the GPU (FP64, mixed) and of the reference CPU path (the
    DavidsonSolver restatement driving the reference loop nest on all host threads)."""
    import torch

    from votca_gb300 import bse_operator as bo
    from votca_gb300.davidson import DavidsonSolver
    from votca_gb300.synthetic import qp_energies, screening_w

    v, c, naux, nmo, roots, seed = 8, 64, 256, 72, 10, 0
    mmn = make_mmn(seed, naux, nmo)
    w = screening_w(seed, naux)
    hqp = np.diag(qp_energies(seed, v, c))
    opt = bo.BSEOperator_Options(homo=v - 1, rpamin=0, qpmin=0, vmin=0, cmax=v + c - 1)
    out = {"workload": "tda_singlet_v8_c64_naux256_roots10"}
    ref = None
    for pname, pr in (("fp64", bo.PRECISION_FP64), ("mixed", bo.PRECISION_MIXED)):
        cx = bo.GpuBSEContext(w, bo.TCMatrix_gwbse(mmn), hqp, opt, precision=pr)
        ds = DavidsonSolver()
        ds.set_tolerance(1e-7)
        ds.set_max_search_space(10 * roots)
        ds.solve(bo.SingletOperator_TDA(cx), roots)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        lam, _ = ds.solve(bo.SingletOperator_TDA(cx), roots)
        out[pname] = {"seconds": time.perf_counter() - t0, "iterations": int(ds.num_iterations()),
                      "info": ds.info()}
        if ref is None:
            ref = lam
        else:
            out[pname]["max_abs_diff_meV_vs_fp64"] = float(np.max(np.abs(lam - ref)) * 1e3)
        cx.close()
    if cpu:
        import oracle
        from oracle.davidson_oracle import DavidsonOracle

        oracle.set_threads(os.cpu_count() or 1)
        prob = oracle.BSEProblem(mmn, w, hqp, v, c)
        d = DavidsonOracle()
        d.set_tolerance(1e-7)
        d.max_search_space = 10 * roots
        t0 = time.perf_counter()
        lam_cpu = d.solve(lambda X: prob.matmul_ref(X, "singlet"), prob.diagonal("singlet"), roots)[0]
        out["cpu_reference"] = {"seconds": time.perf_counter() - t0, "cores": os.cpu_count() or 1,
                                "kind": "port", "iterations": int(d.i_iter),
                                "max_abs_diff_meV_vs_gpu_fp64": float(np.max(np.abs(np.asarray(lam_cpu) - ref)) * 1e3)}
    return out


def solve_only(args):
    """The profiler workload: a warm-up solve, then one timed 20-singlet solve (tolerance 1e-7,
    split precision with the FP64 polish) at the workload shape (--shape to change it)."""
    import torch

    from votca_gb300 import bse_operator as bo
    from votca_gb300.davidson import DavidsonSolver
    from votca_gb300.synthetic import qp_energies, screening_w

    v, c, naux, nmo = V, C, NAUX, NMO
    if args.shape:
        v, c, naux, nmo = (int(x) for x in args.shape.split(","))
    mmn = make_mmn(1, naux, nmo)
    opt = bo.BSEOperator_Options(homo=v - 1, rpamin=0, qpmin=0, vmin=0, cmax=v + c - 1)
    ctx = bo.GpuBSEContext(screening_w(1, naux), bo.TCMatrix_gwbse(mmn), np.diag(qp_energies(1, v, c)), opt,
                           precision=bo.PRECISION_MIXED)
    out = {}
    for rep in ("warmup", "timed"):
        ds = DavidsonSolver()
        ds.set_tolerance(1e-7)
        ds.set_max_search_space(10 * ROOTS)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ds.solve(bo.SingletOperator_TDA(ctx), ROOTS)
        r = ds.result
        out[rep] = {"seconds": time.perf_counter() - t0, "iterations": int(ds.num_iterations()),
                    "polished": int(r.polished), "max_residual": r.max_residual,
                    "polish_seconds": r.seconds_polish, "matvec_seconds": r.seconds_matvec}
    ctx.close()
    print(json.dumps({"workload": f"tda_singlet_v{v}_c{c}_naux{naux}_roots{ROOTS}_solve", **out}))


def product_only(args):
    """A profiler workload: the Hd product (cd = 1 only) of one precision applied twice to k
    vectors at the workload shape (--shape), the second application timed."""
    import torch

    from votca_gb300 import bse_operator as bo
    from votca_gb300.synthetic import qp_energies, screening_w

    v, c, naux, nmo = V, C, NAUX, NMO
    if args.shape:
        v, c, naux, nmo = (int(x) for x in args.shape.split(","))
    prec = {"mixed": bo.PRECISION_MIXED, "sliced": bo.PRECISION_SLICED, "fp64": bo.PRECISION_FP64}[args.product_only]
    k = args.columns
    mmn = make_mmn(1, naux, nmo)
    opt = bo.BSEOperator_Options(homo=v - 1, rpamin=0, qpmin=0, vmin=0, cmax=v + c - 1)
    ctx = bo.GpuBSEContext(screening_w(1, naux), bo.TCMatrix_gwbse(mmn), np.diag(qp_energies(1, v, c)), opt,
                           precision=prec)
    n = v * c
    X = torch.randn((k, n), dtype=torch.float64, device="cuda")
    Y = torch.empty((k, n), dtype=torch.float64, device="cuda")
    op = bo.HdOperator(ctx)
    ms = []
    for _ in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        op.matmul_device(X.data_ptr(), n, k, Y.data_ptr(), n, torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        ms.append((time.perf_counter() - t0) * 1e3)
    ctx.close()
    print(json.dumps({"workload": f"hd_product_{args.product_only}_v{v}_c{c}_naux{naux}_k{k}", "ms": ms}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="auto", choices=["auto", "fp64", "mixed"])
    ap.add_argument("--no-roots", action="store_true", help="skip the time-to-roots solves")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--small", action="store_true", help="C0-sized workload (for profiling captures)")
    ap.add_argument("--shape", default=None, help="v,c,naux,nmo override (profiling captures)")
    ap.add_argument("--molecules", type=int, default=256,
                    help="batched independent molecules (0 skips the batched solve report)")
    ap.add_argument("--batch-threads", type=int, default=16, help="host threads of the batched solve")
    ap.add_argument("--no-full-bse", dest="full_bse", action="store_false",
                    help="skip the full-BSE report (v=128, c=1024, Naux=4096, 32 trial vectors per iteration, "
                         "FP64 polish; about 1.5 minutes, ~110 GB of HBM)")
    ap.add_argument("--no-full-bse-check", dest="full_bse_check", action="store_false",
                    help="skip the independent FP64 evaluation of the full-BSE roots")
    ap.add_argument("--product-only", default=None, choices=["mixed", "sliced", "fp64"],
                    help="profiler workload: the Hd product of that precision, twice, at the workload shape")
    ap.add_argument("--columns", type=int, default=8, help="vectors of --product-only")
    ap.add_argument("--batch-only", action="store_true",
                    help="profiler workload: the cold and the warm lockstep solve of the batched set")
    ap.add_argument("--solve-only", action="store_true",
                    help="one split-precision 20-singlet solve (with its FP64 polish) at the workload shape, "
                         "after one warm-up solve, and nothing else (for profiler captures)")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)
    if args.product_only:
        return product_only(args)
    if args.batch_only:
        print(json.dumps(batched_solve(args.molecules, args.batch_threads, lockstep_only=True)))
        return None
    if args.solve_only:
        return solve_only(args)

    import torch

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from votca_gb300 import _lib
    from votca_gb300 import bse_operator as bo
    from votca_gb300.davidson import DavidsonSolver
    from votca_gb300.synthetic import qp_energies, screening_w

    global V, C, NAUX, NMO, WORKLOAD
    if args.small:
        V, C, NAUX, NMO = 8, 64, 256, 72
    if args.shape:
        V, C, NAUX, NMO = (int(x) for x in args.shape.split(","))
    WORKLOAD = f"tda_singlet_v{V}_c{C}_naux{NAUX}_k{K}"
    L = _lib.load()
    seed = 1  # every replica solves the same seeded problem
    mmn = make_mmn(seed, NAUX, NMO)
    w = screening_w(seed, NAUX)
    hqp = np.diag(qp_energies(seed, V, C))
    Mmn = bo.TCMatrix_gwbse(mmn)
    opt = bo.BSEOperator_Options(homo=V - 1, rpamin=0, qpmin=0, vmin=0, cmax=V + C - 1)
    prec_name = args.precision
    if prec_name == "auto":
        prec_name = "mixed"
    precision = bo.PRECISION_MIXED if prec_name == "mixed" else bo.PRECISION_FP64
    t0 = time.perf_counter()
    ctx = bo.GpuBSEContext(w, Mmn, hqp, opt, precision=precision)
    staging_s = time.perf_counter() - t0
    op = bo.SingletOperator_TDA(ctx)
    dim = V * C

    rng = np.random.default_rng(2)
    Xh = torch.from_numpy(np.asfortranarray(rng.standard_normal((dim, K))).T.copy())  # (K, dim) row-major
    dX = Xh.to("cuda")
    dY = torch.empty_like(dX)
    stream = torch.cuda.current_stream().cuda_stream

    def step():
        op.matmul_device(dX.data_ptr(), dim, K, dY.data_ptr(), dim, stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # per-stage device time (events on the launch stream) for the roofline figure
    _lib.check(L.bse_op_profile(ctx.handle, 1))
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ms = e0.elapsed_time(e1) / args.steps
    clk = clocks.stop()
    import ctypes

    stage_ms = (ctypes.c_double * 12)()
    stage_calls = (ctypes.c_int64 * 12)()
    _lib.check(L.bse_op_profile_read(ctx.handle, stage_ms, stage_calls, 12))
    _lib.check(L.bse_op_profile(ctx.handle, 0))
    ms = max_over_ranks(ms, world, "cuda")

    # e2e through the host-pointer C ABI call with pinned buffers
    Xp = torch.empty((K, dim), dtype=torch.float64).pin_memory()
    Xp.copy_(Xh)
    Yp = torch.empty((K, dim), dtype=torch.float64).pin_memory()
    Xptr = ctypes.cast(Xp.data_ptr(), _lib.c_dp)
    Yptr = ctypes.cast(Yp.data_ptr(), _lib.c_dp)
    for _ in range(1):
        _lib.check(L.bse_op_matmul(ctx.handle, *op.coef, Xptr, dim, K, Yptr, dim))
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        _lib.check(L.bse_op_matmul(ctx.handle, *op.coef, Xptr, dim, K, Yptr, dim))
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e_s = max_over_ranks(e2e_s, world, "cuda")
    # consistency of the two paths
    yd = dY.cpu().numpy()
    rel = float(np.linalg.norm(Yp.numpy() - yd) / np.linalg.norm(yd))

    F = algorithmic_flops(V, C, NAUX, K)
    value = replica_throughput(F, ms * 1e-3, world) / 1e12
    e2e_val = replica_throughput(F, e2e_s, world) / 1e12

    # roofline of the dominant kernel
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    if precision == bo.PRECISION_FP64:
        fp64 = ctypes.c_double()
        _lib.check(L.bse_probe_fp64_tflops(ctypes.byref(fp64)))
        st = 2  # BSE_STAGE_HD_A
        per_launch_ms = stage_ms[st] / max(1, stage_calls[st])
        launches_per_step = stage_calls[st] / max(1, args.steps)
        achieved = hd_stage_a_flops(V, C, NAUX, K) / launches_per_step / (per_launch_ms * 1e-3) / 1e12
        roofline = {"bound": "fp64", "kernel": "dgemm_kernel (Hd c-contraction, FP64 CUDA cores)",
                    "achieved": achieved, "peak": fp64.value, "unit": "TFLOP/s",
                    "frac": achieved / fp64.value,
                    "peak_source": "measured in-run: FP64 FMA register loop (bse_probe_fp64_tflops)",
                    "traffic": None}
    else:
        st = 6  # BSE_STAGE_TC_HD: the c-contraction GEMM of Hd on the tensor cores
        per_launch_ms = stage_ms[st] / max(1, stage_calls[st])
        launches_per_step = stage_calls[st] / max(1, args.steps)
        achieved = hd_stage_a_flops(V, C, NAUX, K) / launches_per_step / (per_launch_ms * 1e-3) / 1e12
        pk = peaks.get("bf16_tflops")
        nprod = 4 if os.environ.get("VGB_TC_PRODUCTS") == "4" else 3
        # DRAM bytes per launch of this kernel: Mcc2 (hi+lo) read once, X read, the S intermediate
        # written; this model matches the ncu capture of the same kernel on a small case
        # (dram__bytes_read.sum + dram__bytes_write.sum of the stage-1 launch at v=32, c=512,
        # Naux=512, k=30)
        kc = -(-C // 64) * 64
        kg = -(-(NAUX * V) // 64) * 64
        per_launch_cols = K / launches_per_step
        traffic = NAUX * C * kc * 4 + per_launch_cols * V * kc * 4 + per_launch_cols * C * kg * 4
        roofline = {"bound": "tensor",
                    "kernel": "tc_gemm_kernel<256,32> (Hd c-contraction, tcgen05 BF16 split products)",
                    "achieved": achieved, "peak": pk / nprod if pk else None,
                    "unit": f"TFLOP/s (FP64-equivalent; {nprod} BF16 products per term)",
                    "frac": achieved / (pk / nprod) if pk else None,
                    "peak_source": f"MEASURED_PEAKS.json bf16_tflops / {nprod} (of measured)",
                    "traffic": traffic, "traffic_source": "bytes per launch, model validated by ncu dram__bytes"}
    stages = {name: {"ms_per_step": stage_ms[i] / args.steps, "launches_per_step": stage_calls[i] / args.steps}
              for i, name in enumerate(["hqp", "hx", "hd_a", "hd_b", "hd2_a", "hd2_b", "tc_hd", "tc_hx",
                                        "tc_hd2", "tc_split", "tc_hd_b", "tc_hd2_b"]) if stage_calls[i]}
    gpu_launches = None
    try:
        gpu_launches = int(sum(stage_calls) / args.steps * args.steps)
    except Exception:
        pass

    line = {
        "metric": "bse_matvec_tflops", "value": value, "unit": "TFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if precision == bo.PRECISION_FP64 else "bf16x3/f64",
        "data": "synthetic (seeded; distributions of the VOTCA GW-BSE workload definition)",
        "config": {"workload": WORKLOAD, "v": V, "c": C, "naux": NAUX, "nmo": NMO, "k": K,
                   "precision": prec_name, "parallelism": f"replicas{world}",
                   "l2": "inputs larger than L2 (staged Mmn blocks > 5 GB)"},
        "e2e": {"value": e2e_val, "unit": "TFLOP/s", "h2d_bytes_per_step": dim * K * 8,
                "d2h_bytes_per_step": dim * K * 8, "matches_device_path_rel": rel},
        "roofline": roofline,
        "flops_per_step": {"algorithmic": F, "reference_algorithm": ref_matvec_flops(V, C, NAUX, K),
                           "note": "value and roofline use the algorithmic count; the reference loop "
                                   "nest executes the second (rows rebuilt on every call)"},
        "stages": stages,
        "staging_seconds": staging_s,
        "clocks": clk,
        "gpu_launches": gpu_launches,
    }
    if rank == 0 and not args.no_roots:
        line["time_to_20_roots"] = roots_report(ctx, precision, w, Mmn, hqp, opt)
        line["c0_time_to_10_roots"] = c0_report(cpu=world == 1 and not args.no_cpu)
    if rank == 0 and (args.molecules > 0 or args.full_bse):
        ctx.close()
    if rank == 0 and args.molecules > 0:
        line["batched"] = batched_solve(args.molecules, args.batch_threads, cpu=world == 1 and not args.no_cpu)
    if rank == 0 and args.full_bse:
        line["full_bse"] = full_bse_report(check=args.full_bse_check, cpu=world == 1 and not args.no_cpu)
    if rank == 0 and world == 1 and not args.no_cpu:
        cb = cpu_baseline(mmn, w, hqp, factorised=True, triplet="time_to_20_roots" in line)
        if "time_to_20_roots" in line:
            cpu_time_to_roots(line["time_to_20_roots"],
                              {"singlets": cb["seconds_per_matvec"],
                               "triplets": cb.get("triplet", {}).get("seconds_per_matvec")})
        cb.pop("seconds_per_matvec", None)
        line["cpu_baseline"] = cb
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
