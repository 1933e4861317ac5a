"""Autotuner for the mixed-precision solvers.  Each knob set is timed on the
workload itself on the device (the library's own CUDA-event solve times)
and the choice is cached in a JSON file keyed by the device and the
workload:

* tune_batch (batched uneven boxes): the FP32 SpMV tile shape (rows per
  tile, pipeline stages), the vector-kernel chunk size and the reliable-
  update interval refine_k;
* tune_mixed (one box): refine_k over 10..50 and the reliable-update drop
  inner_tol;
* tune_multi (many right-hand sides on one box): the stencil SpMM's z steps
  per work item, then refine_k and inner_tol.

The batch search, in detail:

Search (coordinate descent, each timing read from the library's own CUDA
events, results[i].times[4]):

1. SpMV shape: every (rows, stages) the library instantiates, each timed on
   a solve capped at `probe_iters` iterations, so every shape does the same
   work (skipped when the batch runs the FP32 stencil operator, which has
   one shape: the first trial reports it);
2. chunk rows: the same capped solve at the best shape;
3. refine_k: full solves to the tolerance at the best shape and chunk, only
   candidates whose every box converges.

The cache lives in $MFE_TUNE_CACHE, else minife_gb300/_tuning_cache.json.
"""
from __future__ import annotations

import hashlib
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))

SHAPES = [(256, 2), (256, 3), (256, 4), (128, 2), (128, 3), (128, 4)]
# one box: refine_k over 10..50 (every k inner iterations at most between
# reliable updates), crossed with the residual drop that triggers one earlier
SINGLE_REFINE_K = [10, 20, 30, 40, 50]
SINGLE_INNER_TOL = [0.1, 0.01]
# multi-RHS: stencil SpMM z steps per item, then refine_k x inner_tol
MULTI_ZCHUNK = [8, 16, 32, 64]
MULTI_REFINE_K = [25, 50, 100]
MULTI_INNER_TOL = [0.1, 0.01]
CHUNKS = [4096, 8192, 16384, 32768]
REFINE_K = [25, 50, 100, 200]
DEFAULT = {"spmv_rows": 256, "spmv_stages": 2, "chunk_rows": 8192, "refine_k": 50}


def cache_path() -> str:
    return os.environ.get("MFE_TUNE_CACHE", os.path.join(HERE, "_tuning_cache.json"))


def _device_key() -> str:
    import torch
    if not torch.cuda.is_available():
        return "no-gpu"
    p = torch.cuda.get_device_properties(torch.cuda.current_device())
    return "%s/sm%d" % (p.name, p.multi_processor_count)


def signature(dims, precision: str) -> str:
    """Device, precision and the multiset of box dimensions."""
    h = hashlib.sha1(json.dumps(sorted(tuple(int(v) for v in d) for d in dims)).encode())
    return "%s|%s|%s" % (_device_key(), precision, h.hexdigest()[:16])


def _load() -> dict:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(key: str, entry: dict) -> None:
    data = _load()
    data[key] = entry
    path = cache_path()
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def lookup(dims, precision: str = "mixed") -> dict | None:
    return _load().get(signature(dims, precision))


def _best_full(trials, run, log):
    """Time run(cfg) for every cfg of trials (dicts); the fastest whose
    every solve converged wins.  Returns (cfg, seconds, records)."""
    best, best_t, rec = None, None, []
    for cfg in trials:
        t, ok = run(cfg)
        rec.append(dict(cfg, seconds=t, converged=ok))
        if log:
            log("%s: %.4f s%s" % (cfg, t, "" if ok else " (not converged)"))
        if ok and (best_t is None or t < best_t):
            best, best_t = cfg, t
    return best, best_t, rec


def tune_mixed(A, b, tol: float = 1e-8, tol_mode: str = "relative", max_iter: int = 5000,
               reps: int = 2, use_cache: bool = True, log=None) -> dict:
    """Tune the single-box mixed solve of A x = b (A a minife_gb300.CSRMatrix
    of a box): refine_k in SINGLE_REFINE_K x inner_tol in SINGLE_INNER_TOL,
    full solves from x = 0 to the tolerance, best of `reps`.  Returns
    {"refine_k", "inner_tol", "solve_seconds", "cached", ...}."""
    import minife_gb300 as M
    key = signature([A.box], "mixed-single")
    if use_cache:
        hit = _load().get(key)
        if hit is not None:
            return dict(hit, cached=True)
    x = b.new_zeros(b.shape)

    def run(cfg):
        best, ok = None, True
        for _ in range(reps):
            x.zero_()
            r = M.cg_solve(A, b, x, max_iter=max_iter, tol=tol, tol_mode=tol_mode,
                           precision="mixed", refine_k=cfg["refine_k"], inner_tol=cfg["inner_tol"])
            ok = ok and r.status == 0
            best = r.total_time if best is None else min(best, r.total_time)
        return best, ok

    trials = [{"refine_k": k, "inner_tol": it} for k in SINGLE_REFINE_K for it in SINGLE_INNER_TOL]
    best, t, rec = _best_full(trials, run, log)
    if best is None:
        best, t = {"refine_k": SINGLE_REFINE_K[-1], "inner_tol": 0.01}, None
    entry = dict(best, solve_seconds=t, trials=rec)
    if use_cache:
        _store(key, entry)
    return dict(entry, cached=False)


def tune_multi(A, B, X, tol: float = 1e-8, tol_mode: str = "relative", max_iter: int = 5000,
               probe_iters: int = 40, reps: int = 2, use_cache: bool = True, log=None) -> dict:
    """Tune the multi-RHS mixed solve of A X = B (B, X device (n, nrhs)):
    the stencil SpMM's z steps per work item on solves capped at probe_iters
    iterations (the same work for every shape), then refine_k x inner_tol on
    full solves.  The chosen z_chunk is applied to the context.  Returns
    {"z_chunk", "refine_k", "inner_tol", "solve_seconds", "cached", ...}."""
    import minife_gb300 as M
    key = signature([A.box], "mixed-multi%d" % B.shape[1])
    if use_cache:
        hit = _load().get(key)
        if hit is not None:
            M.set_multi_tuning(hit["z_chunk"])
            return dict(hit, cached=True)

    def solve(cfg, cap):
        best, ok = None, True
        for _ in range(reps):
            X.zero_()
            res = M.cg_solve_multi(A, B, X, max_iter=cap or max_iter, tol=0.0 if cap else tol,
                                   tol_mode=tol_mode, precision="mixed",
                                   refine_k=cfg["refine_k"], inner_tol=cfg["inner_tol"])
            ok = ok and all(r.status == 0 for r in res)
            t = res[0].times[4]
            best = t if best is None else min(best, t)
        return best, ok

    cur = {"z_chunk": 32, "refine_k": 50, "inner_tol": 0.01}
    rec = []
    best_t = None
    for zc in MULTI_ZCHUNK:
        M.set_multi_tuning(zc)
        t, _ = solve(dict(cur, z_chunk=zc), probe_iters)
        rec.append(dict(cur, z_chunk=zc, seconds=t, stage="capped"))
        if log:
            log("capped z_chunk=%d: %.4f s" % (zc, t))
        if best_t is None or t < best_t:
            best_t, cur = t, dict(cur, z_chunk=zc)
    M.set_multi_tuning(cur["z_chunk"])
    trials = [dict(cur, refine_k=k, inner_tol=it) for k in MULTI_REFINE_K for it in MULTI_INNER_TOL]
    best, t, rec2 = _best_full(trials, lambda cfg: solve(cfg, 0), log)
    if best is None:
        best, t = cur, None
    entry = dict(best, solve_seconds=t, trials=rec + rec2)
    if use_cache:
        _store(key, entry)
    return dict(entry, cached=False)


def _solve_time(batch, precision, tol, tol_mode, max_iter, refine_k, reps):
    best, res = None, None
    for _ in range(reps):
        _, res = batch.solve(max_iter=max_iter, tol=tol, tol_mode=tol_mode, precision=precision,
                             refine_k=refine_k)
        t = res[0].times[4]
        best = t if best is None else min(best, t)
    return best, res


def tune_batch(batch, precision: str = "mixed", tol: float = 1e-8, tol_mode: str = "relative",
               max_iter: int = 5000, probe_iters: int = 40, reps: int = 2, use_cache: bool = True,
               log=None) -> dict:
    """Tune `batch` (a minife_gb300.Batch) and apply the result to it.
    Returns the chosen configuration with the timings behind it."""
    key = signature(batch.dims, precision)
    if use_cache:
        hit = _load().get(key)
        if hit is not None:
            batch.set_tuning(hit["spmv_rows"], hit["spmv_stages"], hit["chunk_rows"])
            return dict(hit, cached=True)
    say = log or (lambda *a: None)
    cur = dict(DEFAULT)
    trials = []

    op = ["none"]

    def capped(cfg):
        batch.set_tuning(cfg["spmv_rows"], cfg["spmv_stages"], cfg["chunk_rows"])
        t, res = _solve_time(batch, precision, 0.0, tol_mode, probe_iters, cfg["refine_k"], reps)
        op[0] = getattr(res[0], "inner_operator", "none")
        trials.append({"stage": "capped", **cfg, "seconds": t})
        say("capped %s: %.4f s" % (cfg, t))
        return t

    best_t = None
    for rows, stages in SHAPES:
        cfg = dict(cur, spmv_rows=rows, spmv_stages=stages)
        t = capped(cfg)
        if best_t is None or t < best_t:
            best_t, cur = t, cfg
        if op[0] == "stencil":
            break  # the SpMV shape does not apply to the stencil operator
    for chunk in CHUNKS:
        if chunk == cur["chunk_rows"]:
            continue
        cfg = dict(cur, chunk_rows=chunk)
        t = capped(cfg)
        if t < best_t:
            best_t, cur = t, cfg
    batch.set_tuning(cur["spmv_rows"], cur["spmv_stages"], cur["chunk_rows"])
    best_full = None
    if precision == "mixed":
        for k in REFINE_K:
            t, res = _solve_time(batch, precision, tol, tol_mode, max_iter, k, reps)
            ok = all(r.status == 0 for r in res)
            trials.append({"stage": "full", **dict(cur, refine_k=k), "seconds": t, "converged": ok})
            say("full refine_k=%d: %.4f s%s" % (k, t, "" if ok else " (not converged)"))
            if ok and (best_full is None or t < best_full):
                best_full, cur = t, dict(cur, refine_k=k)
    else:
        best_full, _ = _solve_time(batch, precision, tol, tol_mode, max_iter, cur["refine_k"], reps)
    entry = dict(cur, solve_seconds=best_full, inner_operator=op[0], trials=trials)
    if use_cache:
        _store(key, entry)
    return dict(entry, cached=False)
