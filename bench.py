"""Benchmark: branch-site model A lnL+gradient evaluations per second on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--precision fast|fp64] [--ns 64] [--ncodon 5000]

Workload (one "step"): one lnL + analytic-gradient evaluation of a 64-taxon x
5000-codon alignment (seeded model-A simulation: random unrooted tree,
branch lengths ~Exp(0.1), one foreground branch, F3x4 from Dirichlet(5),
kappa=2, w0=0.3, w2=3, p0=0.5, p1=0.3), gradient w.r.t. all 125 branch
lengths, kappa, w0, w2, p0, p1.

* value  -- device-resident throughput: the evaluation's CUDA graphs replayed
            K times with inputs already on the device (CUDA events).
* e2e    -- the same metric through the public API (gb_eval with host arrays:
            host model set-up, host->device parameter copy, device->host result
            and gradient copies inside the timed region).
* roofline -- the dominant kernel class, algorithmic FLOPs / its measured time.
* cpu_baseline -- the reference codeml itself (its CPU build from the staged
            reference sources, oracle/Makefile) on all host cores, one process
            per core, a bounded sample: one step of lfundG plus one forward-
            difference gradient coordinate per process; a CPU lnL+gradient
            costs np+1 lnL evaluations (codeml's forward-difference gradientB).
            Where the reference cannot be built, the oracle port.
--impl reference times the same reference codeml, K steps after W warm-ups,
as the reference arm.
Multi-GPU: replicas only (each rank evaluates its own copy); value sums ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "lnL+gradient evals/sec on 1 GB300 vs plain FP64 GPU & host CPU at |ΔlnL|≤1e-6"
PARAMS = dict(kappa=2.0, omega0=0.3, omega2=3.0, p0=0.5, p1=0.3)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for k, n in enumerate(names):
                if p[5 + k].lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def make_workload(ns: int, ncodon: int, seed: int = 2024):
    from cucodeml_gb300 import api
    from cucodeml_gb300.simulate import simulate
    aln = simulate(ns, ncodon, seed=seed)
    z, fpatt, pi = api.patterns(aln.codons)
    return aln.tree, z, fpatt, pi


# DRAM bytes (read + write) per launch of the persistent split-precision
# kernels from one ncu capture at 32 taxa x 2000 codons (1974 patterns, 62
# contractions, 910811496 contraction FLOPs), profiles/fast_kernels_32x2000.md;
# scaled to another workload by its contraction FLOPs
NCU_TRAFFIC_SMALL = {"prune": 29.09e6 + 68.11e6, "bwd": 87.62e6 + 137.58e6, "gradP": 193.19e6 + 10.66e6}
NCU_FLOPS_SMALL = 910811496.0


def count_flops(lk_tree, z, fpatt):
    """Algorithmic FLOPs of one lnL and one lnL+gradient evaluation.

    Contractions: 2*61^2*npatt per (node, class, internal child) computed by the
    minimal schedule (classes 0,1 at every node, 2a/2b only where a foreground
    branch lies below); P(t): 2*61^3 per unique (branch, omega) pair.
    lnL+gradient = 3 x lnL (forward, adjoint propagation, dlnL/dP)."""
    tree = lk_tree
    ns, nn = tree.ns, tree.nnode
    dirty = np.zeros(nn, dtype=bool)
    for n in tree.postorder():
        for s in tree.sons[n]:
            if tree.label[s] == 1 or dirty[s]:
                dirty[n] = True
    nc = 0
    for a in range(ns, nn):
        ncls = 4 if (dirty[a] or a == tree.root) else 2
        nc += ncls * sum(1 for s in tree.sons[a] if s >= ns)
    npair = sum(3 if tree.label[n] else 2 for n in range(nn) if n != tree.root)
    P = len(fpatt)
    f_contr = 2.0 * 61 * 61 * P * nc
    f_pmat = 2.0 * 61 ** 3 * npair
    return {"contractions": nc, "npair": npair, "flops_prune": f_contr, "flops_pmat": f_pmat,
            "flops_lnL": f_contr + f_pmat, "flops_lnL_grad": 3 * (f_contr + f_pmat),
            "flops_nominal_lnL": 4.0 * (nn - ns - 1) * 2 * 61 * 61 * P}


def fp64_peak_tflops():
    """FP64 GEMM throughput (cuBLAS DGEMM via torch), the FP64 roof of this GPU."""
    import torch
    n = 4096
    a = torch.rand(n, n, dtype=torch.float64, device="cuda")
    b = torch.rand(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = 0.0
    for _ in range(3):
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 2 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    del a, b
    return best


def batched_leg(args, dev):
    """Batched workload: args.batch independent genes (taxa U{12..48}, codons
    log-uniform [100, 3000], per-gene kappa, w0, w2), lnL + gradient of every
    gene per step, one CUDA-graph launch per step; split precision and FP64."""
    from cucodeml_gb300 import api
    from cucodeml_gb300.simulate import simulate_batch
    alns = simulate_batch(args.batch, seed=4)
    genes = []
    for a in alns:
        z, fp, pi = api.patterns(a.codons)
        genes.append((a.tree, z, fp, pi))
    prm = [{"blength": a.tree.branch, "kappa": a.model.kappa, "omega0": a.model.omega0,
            "omega2": a.model.omega2, "p0": a.model.p0, "p1": a.model.p1} for a in alns]
    out = {"genes": args.batch, "patterns": int(sum(len(g[2]) for g in genes)),
           "workload": f"{args.batch} genes, taxa U{{12..48}}, codons log-uniform [100, 3000], lnL+gradient"}
    res = {}
    tuning = None
    if not args.no_tune:
        from cucodeml_gb300 import autotune
        t0 = time.perf_counter()
        tr = autotune.tune_batch(genes, prm, use_cache=False)
        tuning = tr["config"]
        out["autotune"] = {"chosen": tuning, "seconds": round(time.perf_counter() - t0, 1),
                           "candidates": [{"config": t["config"], "ms_per_batch": t.get("ms"),
                                           "agrees": t.get("agrees")} for t in tr["table"]]}
    for prec in ("fast", "fp64"):
        tn = tuning if prec == "fast" else None
        b = api.Batch(genes, precision=prec, device=dev, tuning=tn)
        f, g, st = b.evaluate(prm, grad=True)
        f, g, st = b.evaluate(prm, grad=True)
        res[prec] = (f, g)
        t0 = time.perf_counter()
        for _ in range(args.batch_steps):
            f, g, st = b.evaluate(prm, grad=True)
        e2e_serial = (time.perf_counter() - t0) / args.batch_steps
        ms = b.replay(args.batch_steps, True) / args.batch_steps
        kernels = st.kernels
        b.close()
        # end to end with the genes in two halves whose host set-up and device
        # work overlap (gb_batch_submit / gb_batch_collect), every step a whole
        # lnL + gradient of all genes with its copies in and out
        pb = api.PipelinedBatch(genes, precision=prec, device=dev, tuning=tn)
        pb.evaluate_many([prm] * 2, grad=True)
        t0 = time.perf_counter()
        rp = pb.evaluate_many([prm] * args.batch_steps, grad=True)
        e2e = (time.perf_counter() - t0) / args.batch_steps
        pb.close()
        assert np.max(np.abs(rp[-1][0] - f)) <= 1e-9 * np.max(np.abs(f))
        out[prec] = {"batch_evals_per_s": 1000.0 / ms, "gene_evals_per_s": args.batch * 1000.0 / ms,
                     "ms_per_batch": ms, "e2e_batch_evals_per_s": 1.0 / e2e,
                     "e2e_gene_evals_per_s": args.batch / e2e,
                     "e2e_serial_batch_evals_per_s": 1.0 / e2e_serial, "kernels_per_batch": kernels,
                     "e2e_note": "two half-batches, host set-up of one overlapping the device work of the "
                                 "other (gb_batch_submit / gb_batch_collect); serial: gb_batch_eval"}
    out["speedup_vs_fp64"] = out["fast"]["batch_evals_per_s"] / out["fp64"]["batch_evals_per_s"]
    out["e2e_speedup_vs_fp64"] = out["fast"]["e2e_batch_evals_per_s"] / out["fp64"]["e2e_batch_evals_per_s"]
    out["max_abs_dlnL_vs_fp64"] = float(np.max(np.abs(res["fast"][0] - res["fp64"][0])))
    err = 0.0
    for a, b in zip(res["fp64"][1], res["fast"][1]):
        va = np.concatenate([a["blength"], [a[k] for k in ("kappa", "omega0", "omega2", "p0", "p1")]])
        vb = np.concatenate([b["blength"], [b[k] for k in ("kappa", "omega0", "omega2", "p0", "p1")]])
        err = max(err, float(np.max(np.abs(va - vb) / np.maximum(1.0, np.abs(va)))))
    out["max_grad_rel_err_vs_fp64"] = err
    return out


def max_over_ranks(vals, device):
    """Each value's maximum over the ranks of the process group (the slowest
    replica's times; one all-reduce)."""
    import torch
    t = torch.tensor(list(vals), dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return [float(v) for v in t]


def secondary_leg(fn, *a):
    """A leg beside the headline (BEB, standard errors): its failure is
    reported in its own object and does not take the headline line down."""
    try:
        return fn(*a)
    except Exception as e:  # noqa: BLE001 -- reported, not swallowed
        return {"error": f"{type(e).__name__}: {e}"}


def beb_leg(args, dev, tree, z, fpatt, pi, bl0):
    """Bayes empirical Bayes site analysis of model A (gb_beb, FP64) on the
    bench alignment at the bench parameters: device and end-to-end time of one
    analysis; with the CPU leg, the oracle's BEB on a pattern subset, scaled by
    patterns (every part of the analysis is linear in the pattern count)."""
    from cucodeml_gb300 import api
    lk = api.Likelihood(tree, z, fpatt, pi, precision="fp64", device=dev)
    args_beb = (bl0, PARAMS["kappa"], PARAMS["omega0"], PARAMS["omega2"], PARAMS["p0"], PARAMS["p1"])
    r = lk.beb(*args_beb)
    runs = []
    for _ in range(3):
        t0 = time.perf_counter()
        r = lk.beb(*args_beb)
        runs.append((time.perf_counter() - t0, r["ms_device"]))
    lk.close()
    e2e = min(t for t, _ in runs)
    out = {"workload": f"BEB of model A, {args.ns} taxa x {args.ncodon} codons: f(x_h|w) for 121 omega sets "
                       f"(FP64 prunings) and the 10^4-point grid integral",
           "ms_device": min(d for _, d in runs), "ms_e2e": 1000.0 * e2e, "kernels": r["kernels"],
           "max_abs_post_sum_minus_1": float(np.max(np.abs(r["post"].sum(axis=0) - 1.0))),
           "lnfX": r["lnfX"]}
    if not args.no_cpu:
        from oracle import oracle as O
        S = min(256, len(fpatt))
        pb = O.Problem(tree, np.ascontiguousarray(z[:, :S]), np.ascontiguousarray(fpatt[:S]), pi,
                       nthreads=O.max_threads())
        x = np.concatenate([tree.x_branch_lengths(), [PARAMS["kappa"], PARAMS["p0"], PARAMS["p1"],
                                                      PARAMS["omega0"], PARAMS["omega2"]]])
        t0 = time.perf_counter()
        pb.beb(x, want_lnfw=False)
        dt = time.perf_counter() - t0
        est = dt * len(fpatt) / S
        out["cpu_baseline"] = {"value_ms": 1000.0 * est, "cores": O.max_threads(), "kind": "port",
                               "sample": f"oracle BEB on the first {S} of {len(fpatt)} patterns, "
                                         f"{dt:.2f} s, scaled by patterns"}
        out["e2e_speedup_vs_cpu"] = est / e2e
    return out


def se_leg(args, dev, tree, z, fpatt, pi, cpu_lnL_s=None, cpu_kind="port"):
    """codeml's standard errors (getSE = 1: 2 np likelihood evaluations and
    the outer-product Hessian, gb_se_opg, FP64) at the bench parameters; the
    CPU figure is 2 np oracle lnL evaluations at the CPU leg's measured time."""
    from cucodeml_gb300 import api
    lk = api.Likelihood(tree, z, fpatt, pi, precision="fp64", device=dev)
    x = np.concatenate([tree.x_branch_lengths(), [PARAMS["kappa"], PARAMS["p0"], PARAMS["p1"],
                                                  PARAMS["omega0"], PARAMS["omega2"]]])
    r = lk.se_opg(x)
    t0 = time.perf_counter()
    r = lk.se_opg(x)
    e2e = time.perf_counter() - t0
    lk.close()
    n = len(x)
    out = {"workload": f"standard errors (codeml getSE = 1), {args.ns} taxa x {args.ncodon} codons: "
                       f"{2 * n} FP64 lnL evaluations and the {n} x {n} outer-product Hessian",
           "ms_device": r["ms_device"], "ms_e2e": 1000.0 * e2e, "kernels": r["kernels"],
           "se_all_positive": bool(np.all(r["se"] > 0))}
    if cpu_lnL_s:
        out["cpu_baseline"] = {"value_ms": 1000.0 * 2 * n * cpu_lnL_s, "kind": cpu_kind,
                               "sample": f"2 np = {2 * n} lnL evaluations at the CPU leg's measured "
                                         f"{cpu_lnL_s:.3f} s per evaluation of the whole host"}
        out["e2e_speedup_vs_cpu"] = 2 * n * cpu_lnL_s / e2e
    return out


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def reference_codeml_binary():
    """The reference codeml (CPU build, its own compiler flags) linked with
    oracle/ref_harness.c, built from the staged reference sources by
    oracle/Makefile; None when it cannot be built here."""
    exe = os.path.join(ROOT, "oracle", "_ref", "codeml_timed")
    if not os.path.exists(exe):
        r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "timed"],
                           capture_output=True, text=True)
        if r.returncode != 0 or not os.path.exists(exe):
            return None
    return exe


def reference_cpu(ns: int, ncodon: int, steps: int, warmup: int, procs: int, seed: int = 2024,
                  coords_per_proc: int = 1):
    """The reference's own CPU path on the host cores: `procs` concurrent
    codeml processes (codeml is single-threaded), each on the whole workload
    alignment.  A step of one process is codeml's lfundG at x plus the
    forward differences of `coords_per_proc` gradient coordinates (gradientB's
    forward branch, tools.c:6342-6346), i.e. 1 + coords_per_proc full lnL
    evaluations; the processes take disjoint coordinates.  A forward-difference
    lnL + gradient costs np + 1 lnL evaluations (ming2's first gradient,
    tools.c:6396-6409), so the host's throughput in lnL + gradient evaluations
    per second is procs (1 + coords_per_proc) / (T (np + 1)), T the slowest
    process's mean step time: the np + 1 evaluations spread perfectly over the
    cores (a bound in the reference's favour)."""
    from cucodeml_gb300.simulate import simulate
    from oracle import refcodeml as R
    exe = reference_codeml_binary()
    if exe is None:
        return None
    aln = simulate(ns, ncodon, seed=seed)
    tree = aln.tree
    # codeml's own x space inside ming2 (LASTROUND = 0): p0, p1 through
    # f_and_x (tools.c:1280-1305), p_i = e^{x_i} / (1 + e^{x_0} + e^{x_1})
    p2 = 1.0 - PARAMS["p0"] - PARAMS["p1"]
    x = np.concatenate([tree.x_branch_lengths(), [PARAMS["kappa"], np.log(PARAMS["p0"] / p2),
                                                  np.log(PARAMS["p1"] / p2), PARAMS["omega0"], PARAMS["omega2"]]])
    rows = R.alignment_rows(aln)
    np_ = tree.nbranch + 5
    import tempfile
    dirs, runs = [], []
    t0 = time.perf_counter()
    try:
        for r in range(procs):
            d = tempfile.mkdtemp(prefix="gbref_")
            dirs.append(d)
            R.write_case(d, tree.names, rows, tree.to_newick(), x)
            first = (r * coords_per_proc) % max(1, np_ - coords_per_proc + 1)
            env = dict(os.environ, GBREF_MODE="time", GBREF_STEPS=str(steps), GBREF_WARMUP=str(warmup),
                       GBREF_COORDS=f"{first}:{coords_per_proc}")
            runs.append(subprocess.Popen([exe, "codeml.ctl"], cwd=d, env=env, stdout=subprocess.PIPE,
                                         stderr=subprocess.PIPE, text=True))
        outs = []
        for p in runs:
            o, e = p.communicate()
            if p.returncode != 0:
                raise RuntimeError(f"reference codeml exited {p.returncode}: {e[-500:]}")
            outs.append(R.parse(o))
    finally:
        import shutil
        for d in dirs:
            shutil.rmtree(d, ignore_errors=True)
    wall = time.perf_counter() - t0
    T = max(statistics.mean(o["step_s"]) for o in outs)
    evals = 1 + coords_per_proc
    value = procs * evals / (T * (np_ + 1))
    return {"value": value, "unit": "evals/s", "cores": procs, "kind": "reference",
            "sample": (f"{procs} concurrent reference codeml processes (CPU build, its own -O3 flags; codeml "
                       f"is single-threaded) on the whole {ns} x {ncodon} alignment ({outs[0]['npatt']} "
                       f"patterns); a step of each = codeml's lfundG + {coords_per_proc} forward-difference "
                       f"gradient coordinate(s) = {evals} lnL evaluations, {T:.3f} s (slowest process, mean "
                       f"of {steps}); lnL+gradient = np+1 = {np_ + 1} evaluations spread over the "
                       f"{procs} processes"),
            "step_s": T, "lnL_eval_s": T / evals, "neg_lnL": outs[0]["f0"], "wall_s": wall,
            "npatt": outs[0]["npatt"], "np": np_}


def port_cpu(tree, z, fpatt, pi, threads: int, seconds: float = 12.0, min_evals: int = 2):
    """The oracle port (C restatement of codeml's lfundG, OpenMP over
    patterns) on the host cores, where the reference codeml cannot be built;
    lnL+gradient = (np+1) lnL evaluations."""
    from oracle import oracle as O
    pb = O.Problem(tree, z, fpatt, pi, nthreads=threads)
    x = np.concatenate([tree.x_branch_lengths(), [PARAMS["kappa"], PARAMS["p0"], PARAMS["p1"],
                                                  PARAMS["omega0"], PARAMS["omega2"]]])
    pb.neg_lnL(x)       # warm-up
    t0 = time.perf_counter()
    n = 0
    while n < min_evals or time.perf_counter() - t0 < seconds:
        pb.neg_lnL(x)
        n += 1
        if time.perf_counter() - t0 > 3 * seconds:
            break
    dt = (time.perf_counter() - t0) / n
    np_ = tree.nbranch + 5
    return {"value": 1.0 / ((np_ + 1) * dt), "unit": "evals/s", "cores": threads, "kind": "port",
            "sample": f"{n} lnL evaluations of the workload on {threads} threads, {dt:.3f} s each; "
                      f"lnL+gradient = np+1 = {np_ + 1} lnL evaluations (forward-difference gradientB)",
            "lnL_eval_s": dt}


def reference_gpu_leg(args, neg_lnL_ours):
    """codeml's own CUDA objective CUDA_lfundG on this GPU, through two
    builds of the reference codeml (oracle/Makefile): CuCodeML, the
    reference's cuda-codeml.cu compiled for sm_103a (its kernels,
    cuda-codeml.cu:112-742, schedule 1280-1406), and codeml over this
    library's FP64 drop-in (codeml_adapter.c).  Each is timed inside codeml
    (ref_harness.c, lnL only: codeml's host SetParameters, the four class
    schedules and codeml's mixture included) at the bench point; codeml's
    finite-difference lnL + gradient costs np + 1 of them."""
    from cucodeml_gb300.simulate import simulate
    from oracle import refcodeml as R
    aln = simulate(args.ns, args.ncodon, seed=2024)
    tree = aln.tree
    p2 = 1.0 - PARAMS["p0"] - PARAMS["p1"]
    x = np.concatenate([tree.x_branch_lengths(), [PARAMS["kappa"], np.log(PARAMS["p0"] / p2),
                                                  np.log(PARAMS["p1"] / p2), PARAMS["omega0"], PARAMS["omega2"]]])
    rows = R.alignment_rows(aln)
    np_ = tree.nbranch + 5
    out = {"workload": f"codeml's CUDA_lfundG (lnL only), {args.ns} taxa x {args.ncodon} codons, inside codeml"}
    for key, exe in (("cucodeml_sm103a", "cucodeml"), ("codeml_over_fp64_dropin", "codeml_gb")):
        path = os.path.join(ROOT, "oracle", "_ref", exe)
        if not os.path.exists(path):
            out[key] = {"unavailable": f"oracle/_ref/{exe} not built (reference sources not staged)"}
            continue
        r = R.time_steps(path, tree.names, rows, tree.to_newick(), x, steps=5, warmup=2,
                         env={"GBREF_COORDS": "0:0"})
        T = statistics.median(r["step_s"])
        out[key] = {"lnL_ms": 1000.0 * T, "lnL_evals_per_s": 1.0 / T,
                    "fd_lnL_grad_evals_per_s": 1.0 / ((np_ + 1) * T),
                    "abs_dlnL_vs_ours": abs(r["f0"] - neg_lnL_ours)}
    return out


def codeml_fit_leg(args):
    """codeml's own model-A fit (ming2, codeml.c:683-692) on this GPU from one
    fixed starting point (in.codeml: the simulation's branch lengths x 0.8,
    kappa 1.5, p0 0.6, p1 0.2, w0 0.5, w2 2; codeml's own starting values are
    randomised), three ways: ming2 with finite-difference gradients
    (gradientB, tools.c:6326-6350) of CuCodeML's CUDA_lfundG (the reference's
    GPU path, cuda-codeml.cu for sm_103a); the same over this library's FP64
    drop-in; and ming2 driven by the drop-in's analytic gradient (GB_dfun, the
    one-argument change at codeml.c:688).  Per run: ming2's own wall time,
    rounds and lnL calls (ref_harness.c), the lnL reached and the whole
    codeml run's wall time (reading, initial estimates, NEB / BEB output
    included)."""
    import tempfile
    from cucodeml_gb300.simulate import simulate
    from oracle import refcodeml as R
    aln = simulate(args.fit_ns, args.fit_ncodon, seed=2024)
    tree = aln.tree
    rows = R.alignment_rows(aln)
    p0, p1 = 0.6, 0.2
    x0 = np.concatenate([tree.x_branch_lengths() * 0.8, [1.5, np.log(p0 / (1 - p0 - p1)),
                                                        np.log(p1 / (1 - p0 - p1)), 0.5, 2.0]])
    out = {"workload": f"codeml model-A fit (ming2), {args.fit_ns} taxa x {args.fit_ncodon} codons, seed 2024, "
                       "fixed start"}
    for key, exe, mode in (("cucodeml_fd", "cucodeml", None), ("dropin_fd", "codeml_gb", None),
                           ("dropin_dfun", "codeml_gb", "dfun")):
        path = os.path.join(ROOT, "oracle", "_ref", exe)
        if not os.path.exists(path):
            out[key] = {"unavailable": f"oracle/_ref/{exe} not built (reference sources not staged)"}
            continue
        env = {k: v for k, v in os.environ.items() if not k.startswith("GBREF_")}
        if mode:
            env["GBREF_MODE"] = mode
        with tempfile.TemporaryDirectory() as d:
            R.write_case(d, tree.names, rows, tree.to_newick(), x0)
            t0 = time.perf_counter()
            r = subprocess.run([path, "codeml.ctl"], cwd=d, capture_output=True, text=True, env=env,
                               timeout=args.fit_timeout)
            wall = time.perf_counter() - t0
            if r.returncode != 0:
                out[key] = {"error": f"exit {r.returncode}: {r.stderr[-300:]}"}
                continue
            with open(os.path.join(d, "out.txt")) as f:
                txt = f.read()
        m = re.search(r"lnL\(ntime:\s*\d+\s+np:\s*(\d+)\):\s*(-?\d+\.\d+)", txt)
        g = re.search(r"GBREF_MING2 (\S+) (\d+) (\d+)", r.stderr)
        rounds = int(g.group(2)) if g else None
        out[key] = {"ming2_s": float(g.group(1)) if g else None,
                    # ming2 sets its round counter to maxround (10000) when it stops on line-search failure
                    "ming2_rounds": rounds if rounds is not None and rounds < 10000 else "stopped on line-search failure",
                    "lnL_calls": int(g.group(3)) if g else None, "lnL": float(m.group(2)) if m else None,
                    "np": int(m.group(1)) if m else None, "codeml_wall_s": wall}
    a, b = out.get("cucodeml_fd", {}), out.get("dropin_dfun", {})
    if a.get("ming2_s") and b.get("ming2_s"):
        out["ming2_speedup_dfun_vs_cucodeml_fd"] = a["ming2_s"] / b["ming2_s"]
    return out


def checkpoint_leg(args, dev):
    """Device memory of an FP64 lnL + gradient evaluation at 256 taxa x 20000
    codons with the checkpointed adjoint off and on (GB_TUNE_CHECKPOINT:
    edge messages recomputed per tree level in the reverse sweep), its time,
    and that both give the same lnL and gradient."""
    import torch
    from cucodeml_gb300 import api
    from cucodeml_gb300.simulate import simulate
    aln = simulate(256, 20000, seed=2024)
    z, fpatt, pi = api.patterns(aln.codons)
    tree = aln.tree
    out = {"workload": f"FP64 lnL+gradient, 256 taxa x 20000 codons ({len(fpatt)} patterns)"}
    res = {}
    for ck in (0, 1):
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        lk = api.Likelihood(tree, z, fpatt, pi, precision="fp64", device=dev, tuning={"checkpoint": ck})
        r = lk.evaluate(tree.branch, grad=True, **PARAMS)
        torch.cuda.synchronize()
        used = free0 - torch.cuda.mem_get_info()[0]
        ms = lk.replay(3, True) / 3
        g = np.concatenate([r.grad["blength"], [r.grad[k] for k in ("kappa", "omega0", "omega2", "p0", "p1")]])
        res[ck] = (r.neg_lnL, g)
        out["on" if ck else "off"] = {"device_GB": used / 1e9, "ms_per_eval": ms}
        lk.close()
    out["bit_identical"] = bool(res[0][0] == res[1][0] and np.array_equal(res[0][1], res[1][1]))
    out["memory_ratio"] = out["on"]["device_GB"] / out["off"]["device_GB"]
    return out


def alt_null_leg(args, dev):
    """Model A against its null (w2 = 1) at 256 taxa x 20000 codons: both fits
    by bounded L-BFGS-B driven by the split-precision path's lnL + adjoint
    gradient (optimize.alt_null), then continued with the FP64 path from those
    maxima; wall time, calls, lnL, LRT and the agreement of the two paths.
    codeml's own route, ming2 with finite-difference gradients, costs np + 1
    lnL evaluations per gradient: timed here per evaluation on the FP64 path
    (the lnL codeml would get over the drop-in)."""
    from cucodeml_gb300 import api, optimize
    from cucodeml_gb300.simulate import simulate
    aln = simulate(256, 20000, seed=2025)
    z, fpatt, pi = api.patterns(aln.codons)
    tree = aln.tree
    out = {"workload": f"model A vs null, 256 taxa x 20000 codons ({len(fpatt)} patterns), seed 2025"}
    t0 = time.perf_counter()
    r = optimize.alt_null(tree, z, fpatt, pi, precision="fast")
    t_fast = time.perf_counter() - t0
    t0 = time.perf_counter()
    p = optimize.alt_null(tree, z, fpatt, pi, precision="fp64", x0_alt=r["alt"]["x"], x0_null=r["null"]["x"])
    t_pol = time.perf_counter() - t0
    for name, res, secs in (("split_precision", r, t_fast), ("fp64_continued", p, t_pol)):
        out[name] = {"lnL_alt": res["alt"]["lnL"], "lnL_null": res["null"]["lnL"], "LRT": res["LRT"],
                     "p_mixture": res["p_mixture"], "calls": res["alt"]["calls"] + res["null"]["calls"],
                     "wall_s": secs, "omega2": res["alt"]["omega2"]}
    out["abs_dlnL_alt_paths"] = abs(r["alt"]["lnL"] - p["alt"]["lnL"])
    out["abs_dlnL_null_paths"] = abs(r["null"]["lnL"] - p["null"]["lnL"])
    lk = api.Likelihood(tree, z, fpatt, pi, precision="fp64", device=dev)
    x = np.asarray(p["alt"]["x"])
    lk.evaluate_x(x, lastround=False)
    t0 = time.perf_counter()
    for _ in range(5):
        lk.evaluate_x(x, lastround=False)
    per = (time.perf_counter() - t0) / 5
    lk.close()
    out["fd_gradient_on_this_gpu"] = {"lnL_eval_s": per, "np": len(x), "seconds_per_fd_gradient": per * (len(x) + 1),
                                      "note": "codeml's forward-difference gradient = np + 1 FP64 lnL evaluations"}
    return out


def workload_config(ns: int, ncodon: int) -> dict:
    """The config both arms report (identical dicts)."""
    return {"workload": f"lnL+gradient, {ns} taxa x {ncodon} codons, branch-site model A "
                        f"(seeded simulation, seed 2024)",
            "l2": "working set per evaluation > L2 (no flush needed)"}


def run_reference(args):
    """The reference arm: the reference codeml's own CPU lnL + gradient
    (lfundG, forward-difference gradientB) on all host cores; the oracle port
    when the reference cannot be built on this machine."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    procs = host_cores()
    ref = reference_cpu(args.ns, args.ncodon, args.steps, args.warmup, procs)
    if ref is None:
        from cucodeml_gb300.simulate import simulate
        from oracle import oracle as O
        aln = simulate(args.ns, args.ncodon, seed=2024)
        z, fpatt, pi = O.patterns(aln.codons)
        tree = aln.tree
        pb = O.Problem(tree, z, fpatt, pi, nthreads=procs)
        x = np.concatenate([tree.x_branch_lengths(), [PARAMS["kappa"], PARAMS["p0"], PARAMS["p1"],
                                                      PARAMS["omega0"], PARAMS["omega2"]]])
        for _ in range(args.warmup):
            pb.neg_lnL(x)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            pb.neg_lnL(x)
        dt = (time.perf_counter() - t0) / args.steps
        np_ = tree.nbranch + 5
        ref = {"value": 1.0 / ((np_ + 1) * dt), "unit": "evals/s", "cores": procs, "kind": "port",
               "sample": f"reference codeml not buildable here: the oracle port, one lnL evaluation per "
                         f"step ({dt:.3f} s) on {procs} threads; lnL+gradient = np+1 = {np_ + 1} evaluations",
               "step_s": dt}
    value = ref["value"]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * ref["step_s"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded model-A simulation, seed 2024)",
        "config": workload_config(args.ns, args.ncodon),
        "cpu_baseline": {k: ref[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="best", choices=["best", "fast", "fp64"])
    ap.add_argument("--ns", type=int, default=64)
    ap.add_argument("--ncodon", type=int, default=5000)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-beb", action="store_true", help="skip the Bayes empirical Bayes leg")
    ap.add_argument("--batch", type=int, default=512, help="genes in the batched leg (0: skip it)")
    ap.add_argument("--batch-steps", type=int, default=3)
    ap.add_argument("--no-tune", action="store_true", help="batched leg: skip the autotuner (library defaults)")
    ap.add_argument("--no-refgpu", action="store_true", help="skip the reference-GPU (CuCodeML) leg")
    ap.add_argument("--no-ckpt", action="store_true", help="skip the checkpointed-adjoint memory leg")
    ap.add_argument("--no-altnull", action="store_true", help="skip the 256 x 20000 model A vs null fits")
    ap.add_argument("--no-fit", action="store_true",
                    help="skip codeml's own fit over CuCodeML and over the drop-in (finite differences / GB_dfun)")
    ap.add_argument("--fit-ns", type=int, default=24)
    ap.add_argument("--fit-ncodon", type=int, default=600)
    ap.add_argument("--fit-timeout", type=float, default=900.0)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)

    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    dev = local if torch.cuda.is_available() else 0
    torch.cuda.set_device(dev)

    from cucodeml_gb300 import api
    tree, z, fpatt, pi = make_workload(args.ns, args.ncodon)
    fl = count_flops(tree, z, fpatt)
    precision = "fp64" if args.precision in ("best", "fp64") else "fast"
    if args.precision == "best":
        try:   # the split-precision path when this build has it, else FP64
            probe = api.Likelihood(tree, z, fpatt, pi, precision="fast", device=dev)
            probe.evaluate(tree.branch, grad=True, **PARAMS)
            probe.close()
            precision = "fast"
        except Exception:
            precision = "fp64"
    lk = api.Likelihood(tree, z, fpatt, pi, precision=precision, device=dev)
    bl0 = tree.branch.copy()
    rng = np.random.default_rng(7)

    def step_params(i):
        return bl0 * (1.0 + 0.01 * rng.standard_normal(bl0.shape)).clip(0.5, 1.5)

    # warm-up through the public API (builds the graphs)
    for i in range(args.warmup):
        r = lk.evaluate(step_params(i), grad=True, **PARAMS)
    # ---- e2e: public API with host buffers, K steps
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    h2d = d2h = 0.0
    with ClockSampler(dev) as clk:
        t0 = time.perf_counter()
        for i in range(args.steps):
            r = lk.evaluate(step_params(i), grad=True, **PARAMS)
            h2d += r.h2d_bytes
            d2h += r.d2h_bytes
        torch.cuda.synchronize()
        e2e_s = time.perf_counter() - t0
        # ---- value: device-resident replay of the evaluation's graphs
        for _ in range(args.warmup):
            lk.replay(1, True)
        dev_ms = lk.replay(args.steps, True)
    kernels_per_eval = r.kernels
    if ws > 1:
        dev_ms, e2e_s = max_over_ranks([dev_ms, e2e_s], "cuda")
    value = ws * args.steps / (dev_ms * 1e-3)
    e2e_value = ws * args.steps / e2e_s

    # ---- per-kernel-class times (outside the timed region)
    prof = lk.profile(3, True)
    tot = sum(v[0] for v in prof.values())
    cls_flops = {"prune": fl["flops_prune"], "bwd": fl["flops_prune"], "gradP": fl["flops_prune"],
                 "pmat": fl["flops_pmat"], "gradH": 2 * fl["flops_pmat"]}
    top = max(prof, key=lambda k: prof[k][0])
    top_ms_per_eval = prof[top][0] / 3
    achieved = cls_flops.get(top, 0.0) / (top_ms_per_eval * 1e-3) / 1e12
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    if precision == "fp64":
        peak = fp64_peak_tflops()
        roof = {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak if peak else None, "traffic": None,
                "peak_source": "cuBLAS DGEMM 4096^3 measured in this run (FP64 pipe; no FP64 entry "
                               "in the measured-peaks file)"}
    else:
        peak = peaks.get("bf16_tflops", 1928.4)
        roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "traffic": None,
                "peak_source": "bf16_tflops of measured" if peaks else "fallback"}
    if precision != "fp64":
        # executed tensor work of the digit-plane contractions (not algorithmic):
        # NS = 8 forward planes -> 36 digit pairs, NB = 7 adjoint planes -> 28,
        # over 64 x 64 padded states; dlnL/dP packs two planes per M = 128 tile:
        # 16 tiles per K step = 32 plane pairs for an internal child (28 kept
        # levels + 4 beyond them; a tip's one-hot product executes 8)
        pairs = {"prune": 36, "bwd": 28, "gradP": 32}
        if top in pairs:
            ex = cls_flops[top] * pairs[top] * (64.0 * 64.0) / (61.0 * 61.0)
            roof["executed_tensor_tflops"] = ex / (top_ms_per_eval * 1e-3) / 1e12
            roof["executed_tensor_frac"] = roof["executed_tensor_tflops"] / peak
        roof["limiter"] = ("SIMT work around the MMAs (cutting operands into digit planes, level "
                           "read-outs, double-float products), one 16-warp CTA per SM (see profiles/)")
        if top in NCU_TRAFFIC_SMALL:
            roof["traffic"] = NCU_TRAFFIC_SMALL[top] * fl["flops_prune"] / NCU_FLOPS_SMALL
            roof["traffic_source"] = ("ncu dram__bytes_read+write of the same kernel at 32 taxa x 2000 codons, "
                                      "scaled by contraction work")
    roof.update({"kernel": top, "share": prof[top][0] / tot if tot else None,
                 "flops_per_eval": cls_flops.get(top, 0.0), "ms_per_eval": top_ms_per_eval,
                 "classes_ms_per_eval": {k: v[0] / 3 for k, v in prof.items()}})

    line = {
        "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if precision == "fp64" else "f64+split",
        "data": "synthetic (seeded model-A simulation, seed 2024)",
        "config": workload_config(args.ns, args.ncodon),
        "workload_detail": {"npatt": int(len(fpatt)), "np": tree.nbranch + 5, "precision": precision,
                            "parallelism": f"replicas x{ws}", "flops_lnL_grad_alg": fl["flops_lnL_grad"],
                            "flops_nominal_lnL": fl["flops_nominal_lnL"]},
        "roofline": roof,
        "e2e": {"value": e2e_value, "unit": "evals/s", "h2d_bytes_per_step": h2d / args.steps,
                "d2h_bytes_per_step": d2h / args.steps},
        "clocks": clk.summary(),
        "gpu_launches": int(kernels_per_eval * args.steps),
        "achieved_tflops_alg": fl["flops_lnL_grad"] * args.steps / (dev_ms * 1e-3) / 1e12,
    }
    # same lnL+gradient through the FP64 drop-in, for the speed-up of the fast path
    if precision == "fast":
        lk64 = api.Likelihood(tree, z, fpatt, pi, precision="fp64", device=dev)
        for i in range(args.warmup):
            r64 = lk64.evaluate(step_params(i), grad=True, **PARAMS)
        ms64 = lk64.replay(max(3, args.steps // 4), True) / max(3, args.steps // 4)
        rf = lk.evaluate(bl0, grad=True, **PARAMS)
        r64 = lk64.evaluate(bl0, grad=True, **PARAMS)
        g64 = np.concatenate([r64.grad["blength"], [r64.grad[k] for k in ("kappa", "omega0", "omega2", "p0", "p1")]])
        gf = np.concatenate([rf.grad["blength"], [rf.grad[k] for k in ("kappa", "omega0", "omega2", "p0", "p1")]])
        line["fp64_value"] = 1000.0 / ms64
        line["speedup_vs_fp64"] = line["value"] / line["fp64_value"]
        line["abs_dlnL_vs_fp64"] = abs(rf.neg_lnL - r64.neg_lnL)
        line["grad_rel_err_vs_fp64"] = float(np.max(np.abs(gf - g64) / np.maximum(1.0, np.abs(g64))))
        lk64.close()
    if args.batch > 0:
        line["batched"] = batched_leg(args, dev)
    if not args.no_beb:
        line["beb"] = secondary_leg(beb_leg, args, dev, tree, z, fpatt, pi, bl0)
    cpu_lnL_s, cpu_kind = None, "port"
    if rank == 0 and not args.no_cpu:
        procs = host_cores()
        ref = reference_cpu(args.ns, args.ncodon, 1, 0, procs)
        if ref is None:
            from oracle import oracle as O
            ref = port_cpu(tree, z, fpatt, pi, O.max_threads())
            cpu_lnL_s = ref["lnL_eval_s"]
        else:
            cpu_lnL_s = ref["lnL_eval_s"] / procs      # evaluations spread over the processes
            ref["abs_dlnL_vs_ours"] = abs(ref["neg_lnL"] - lk.evaluate(bl0, grad=False, **PARAMS).neg_lnL)
        cpu_kind = ref["kind"]
        line["cpu_baseline"] = {k: ref[k] for k in ("value", "unit", "cores", "kind", "sample")
                                if k in ref}
        if "abs_dlnL_vs_ours" in ref:
            line["cpu_baseline"]["abs_dlnL_vs_ours"] = ref["abs_dlnL_vs_ours"]
    if not args.no_beb:
        line["se"] = secondary_leg(se_leg, args, dev, tree, z, fpatt, pi, cpu_lnL_s, cpu_kind)
    if not args.no_altnull:
        line["alt_null"] = secondary_leg(alt_null_leg, args, dev)
    if not args.no_ckpt:
        line["checkpoint"] = secondary_leg(checkpoint_leg, args, dev)
    if not args.no_refgpu:
        line["reference_gpu"] = secondary_leg(reference_gpu_leg, args,
                                              lk.evaluate(bl0, grad=False, **PARAMS).neg_lnL)
    if not args.no_fit:
        line["codeml_fit"] = secondary_leg(codeml_fit_leg, args)
    lk.close()
    if rank == 0:
        print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
