"""Autotuner for the block-RPCholesky block size and the batched-calibration
work-item size.

Choices are measured, not modelled: each candidate runs on the caller's own
data (a row prefix for the factorisation, a sample of the batch for the
calibration), timed with CUDA events on the current stream after one untimed
run, and the fastest wins.  Results are cached per problem class
(d, N octave, k bucket) in memory and, when ``KEVD_AUTOTUNE_CACHE`` names a
file, in that JSON file.
"""
from __future__ import annotations

import json
import math
import os
import threading

import numpy as np
import torch

from . import api

_lock = threading.Lock()
_cache: dict[str, dict] = {}
_loaded = False


def _path():
    return os.environ.get("KEVD_AUTOTUNE_CACHE")


def _load():
    global _loaded
    if _loaded:
        return
    _loaded = True
    p = _path()
    if p and os.path.exists(p):
        try:
            with open(p) as f:
                _cache.update(json.load(f))
        except (OSError, ValueError):
            pass


def _store():
    p = _path()
    if not p:
        return
    tmp = p + ".tmp"
    with open(tmp, "w") as f:
        json.dump(_cache, f, indent=1, sort_keys=True)
    os.replace(tmp, p)


def _timed(fn, reps: int = 2) -> float:
    fn()
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    best = float("inf")
    for _ in range(reps):
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return best


def block_key(N: int, d: int, k: int) -> str:
    return f"rpchol/d{d}/n{int(math.log2(max(N, 2)))}/k{(k + 255) // 256}"


def tune_block(ctx: api.Context, X: torch.Tensor, scale: float, k: int, candidates=(16, 32, 64, 128, 256),
               probe_rows: int = 131072, probe_k: int = 512) -> dict:
    """Block size b for a mixed-precision factorisation of X to rank k: each
    candidate factorises the first ``probe_rows`` rows to rank
    ``min(k, probe_k)``; the time per accepted column decides."""
    N, d = X.shape
    key = block_key(N, d, k)
    with _lock:
        _load()
        if key in _cache:
            return dict(_cache[key], cached=True)
    Xp = X[: min(N, probe_rows)].contiguous()
    kp = int(min(k, probe_k, Xp.shape[0]))
    times = {}
    for b in candidates:
        if b > kp:
            continue
        res = {}

        def run(b=b):
            res["f"] = api.rpcholesky(ctx, Xp, scale, k_max=kp, block=b, seed=1, precision="mixed")

        ms = _timed(run)
        times[int(b)] = ms / max(1, res["f"].rank)
    best = min(times, key=times.get)
    entry = {"block": best, "ms_per_column": times, "probe_rows": int(Xp.shape[0]), "probe_k": kp}
    with _lock:
        _cache[key] = entry
        _store()
    return dict(entry, cached=False)


def tune_calibration_items(ctx: api.Context, Xs, scales_list, candidates=(0, 4, 32, 256),
                           sample_jobs: int = 8, max_rows: int = 40000) -> dict:
    """Work-item size (tiles per item, 0 = automatic) of the batched
    calibration, timed on the largest ``sample_jobs`` datasets cut to
    ``max_rows`` rows."""
    order = np.argsort([-X.shape[0] for X in Xs])[:sample_jobs]
    sX = [Xs[i][:max_rows].contiguous() for i in order]
    ss = [scales_list[i] for i in order]
    key = "calib/" + "/".join(f"{X.shape[0]}x{X.shape[1]}" for X in sX)
    with _lock:
        _load()
        if key in _cache:
            return dict(_cache[key], cached=True)
    times = {int(c): _timed(lambda c=c: api.calibrate_batched(ctx, sX, ss, tiles_per_item=int(c))) for c in candidates}
    best = min(times, key=times.get)
    entry = {"tiles_per_item": best, "ms": times}
    with _lock:
        _cache[key] = entry
        _store()
    return dict(entry, cached=False)
