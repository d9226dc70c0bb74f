"""Autotuner of the split-precision path's kernel configuration.

It times candidate configurations (gb_tune knobs: contraction kernel, tile
schedule, patterns per dlnL/dP partial, task order of a batch) on the caller's
own workload, keeps the fastest whose lnL and gradient agree with the first
candidate's, and caches the choice in a JSON file keyed by the GPU and the
workload's shape, so that later runs on the same kind of workload reuse it.

The reference has no counterpart (codeml's GPU module has a fixed schedule).
"""
from __future__ import annotations

import json
import os
import time

import numpy as np

from . import api

#: candidates for batches; the first is the library default and the reference
BATCH_CANDIDATES = [
    {"mma": 1, "persist": 1, "gchunk": 2048, "order": 0},
    {"mma": 1, "persist": 1, "gchunk": 1024, "order": 0},
    {"mma": 1, "persist": 1, "gchunk": 4096, "order": 0},
    {"mma": 1, "persist": 1, "gchunk": 2048, "order": 2},
    {"mma": 1, "persist": 1, "gchunk": 2048, "order": 1},
    {"mma": 1, "persist": 0, "gchunk": 2048},
    {"mma": 0, "persist": 0, "gchunk": 2048},
]

#: candidates for a single alignment
SINGLE_CANDIDATES = [
    {"mma": 1, "persist": 1, "gchunk": 2048},
    {"mma": 1, "persist": 1, "gchunk": 1024},
    {"mma": 1, "persist": 1, "gchunk": 4096},
    {"mma": 1, "persist": 0, "gchunk": 2048},
    {"mma": 0, "persist": 0, "gchunk": 2048},
]


def default_cache_path() -> str:
    p = os.environ.get("GBCODEML_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "cucodeml_gb300", "autotune.json")


def gpu_name() -> str:
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.get_device_name(0)
    except Exception:
        pass
    return "cuda"


def signature(shapes, kind: str) -> str:
    """Cache key: GPU, kind (batch / single) and the workload's shape in
    coarse buckets (gene count, taxa range, total patterns to 2 significant
    digits)."""
    ns = [s[0] for s in shapes]
    npatt = sum(s[1] for s in shapes)
    tot = float(f"{npatt:.2g}")
    return f"{gpu_name()}|{kind}|genes={len(shapes)}|taxa={min(ns)}-{max(ns)}|patterns~{tot:g}"


def _load(path: str) -> dict:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path: str, key: str, entry: dict) -> None:
    d = _load(path)
    d[key] = entry
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(d, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def _gvec(g) -> np.ndarray:
    return np.concatenate([g["blength"], [g[k] for k in ("kappa", "omega0", "omega2", "p0", "p1")]])


def _agree(ref, got, lnl_tol: float, grad_tol: float) -> bool:
    (f0, g0), (f1, g1) = ref, got
    if not np.all(np.abs(np.asarray(f0) - np.asarray(f1)) <= lnl_tol):
        return False
    for a, b in zip(g0, g1):
        va, vb = _gvec(a), _gvec(b)
        if np.max(np.abs(va - vb) / np.maximum(1.0, np.abs(va))) > grad_tol:
            return False
    return True


def choose(key: str, candidates, run, cache_path: str | None = None, use_cache: bool = True,
           lnl_tol: float = 1e-6, grad_tol: float = 1e-5) -> dict:
    """Time run(cfg) -> (ms, (lnL values, gradients)) for every candidate and
    return {"config", "ms", "table", "key", "cached"}.  A candidate whose
    results disagree with the first candidate's (beyond the split-precision
    tolerances) is reported but never chosen."""
    path = cache_path or default_cache_path()
    if use_cache:
        hit = _load(path).get(key)
        if hit:
            return dict(hit, cached=True)
    table, ref = [], None
    for cfg in candidates:
        t0 = time.perf_counter()
        try:
            ms, res = run(cfg)
        except Exception as e:          # a configuration the library refuses
            table.append({"config": cfg, "ms": None, "error": str(e)})
            continue
        ok = True if ref is None else _agree(ref, res, lnl_tol, grad_tol)
        if ref is None:
            ref = res
        table.append({"config": cfg, "ms": ms, "agrees": ok, "setup_s": time.perf_counter() - t0})
    good = [r for r in table if r.get("ms") is not None and r.get("agrees")]
    if not good:
        raise RuntimeError("autotune: no candidate ran")
    best = min(good, key=lambda r: r["ms"])
    entry = {"config": best["config"], "ms": best["ms"], "table": table, "key": key}
    _store(path, key, entry)
    return dict(entry, cached=False)


def tune_batch(genes, params, precision: str = "fast", candidates=None, reps: int = 2, **kw) -> dict:
    """genes: list of (tree, z, fpatt, pi); params: per-gene parameter dicts
    (as for Batch.evaluate).  Times lnL + gradient of the whole batch."""
    shapes = [(g[0].ns, len(g[2])) for g in genes]

    def run(cfg):
        b = api.Batch(genes, precision=precision, tuning=cfg)
        try:
            b.evaluate(params, grad=True)
            f, g, _ = b.evaluate(params, grad=True)
            ms = b.replay(reps, True) / reps
            return ms, (f, g)
        finally:
            b.close()

    return choose(signature(shapes, "batch-" + precision), candidates or BATCH_CANDIDATES, run, **kw)


def tune_single(tree, z, fpatt, pi, args, precision: str = "fast", candidates=None, reps: int = 5,
                **kw) -> dict:
    """args: (blength, kappa, omega0, omega2, p0, p1) as for Likelihood.evaluate."""

    def run(cfg):
        lk = api.Likelihood(tree, z, fpatt, pi, precision=precision, tuning=cfg)
        try:
            lk.evaluate(*args, grad=True)
            r = lk.evaluate(*args, grad=True)
            ms = lk.replay(reps, True) / reps
            return ms, ([r.neg_lnL], [r.grad])
        finally:
            lk.close()

    return choose(signature([(tree.ns, len(fpatt))], "single-" + precision), candidates or SINGLE_CANDIDATES,
                  run, **kw)
