"""Autotuner for the batched LU schedule.

The batched solver runs one persistent kernel per size bucket inside one CUDA
graph.  Which bucket edges, threads per CTA, panel widths and CTA counts are
fastest depends on the batch's size distribution, so this module searches
them by timing the real solve on the device and caches the winner, keyed by a
signature of the distribution -- the role LinearSolve.jl's autotuner plays for
its size buckets (lib/LinearSolveAutotune, preferences read back at load
time by src/preferences.jl / src/default.jl:354-396).

    sched = tune(ctx, sizes, precision="fp32")      # measures, caches, returns
    apply(ctx, batch_handle, sched)                  # gblu_batch_schedule
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import os
import time

import numpy as np

from . import _lib
from ._cuda import DeviceMatrix, Event

# (threads per CTA, panel width) variants compiled into libgblu
VARIANTS = [(64, 8), (128, 8), (128, 16), (256, 8), (256, 16), (512, 16)]
EDGE_SETS = [[256], [64, 256], [128, 256], [64, 128, 256], [32, 96, 256], [48, 96, 160, 256]]
PRECISIONS = {"fp64": _lib.GBLU_FP64, "fp32": _lib.GBLU_FP32}


def cache_path() -> str:
    p = os.environ.get("GBLU_AUTOTUNE_FILE")
    if p:
        return p
    base = os.environ.get("XDG_CACHE_HOME", os.path.join(os.path.expanduser("~"), ".cache"))
    return os.path.join(base, "gblu", "autotune.json")


def signature(sizes, precision: str) -> str:
    """Histogram of n in 16-wide bins plus the count, hashed: batches with the
    same distribution share a schedule."""
    sizes = np.asarray(sizes, dtype=np.int64)
    hist = np.bincount(np.minimum(sizes // 16, 16), minlength=17)
    frac = np.round(hist / max(len(sizes), 1), 2)
    key = f"{precision}|{len(sizes) // 1000}k|" + ",".join(f"{x:.2f}" for x in frac)
    return hashlib.sha1(key.encode()).hexdigest()[:16]


def _load_cache() -> dict:
    try:
        with open(cache_path()) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def _store_cache(entries: dict) -> None:
    path = cache_path()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + f".{os.getpid()}.tmp"
    with open(tmp, "w") as fh:
        json.dump(entries, fh, indent=1, sort_keys=True)
    os.replace(tmp, path)


def apply(ctx, handle, sched: dict) -> None:
    edges = np.array(sched["upper"], dtype=np.int32)
    thr = np.array(sched["threads"], dtype=np.int32)
    pan = np.array(sched["panel"], dtype=np.int32)
    ctas = np.array(sched.get("ctas", [0] * len(edges)), dtype=np.int32)
    _lib.check(ctx.lib.gblu_batch_schedule(ctx.handle, handle, len(edges), edges.ctypes.data,
                                           thr.ctypes.data, pan.ctypes.data, ctas.ctypes.data),
               ctx.handle)


def _time_solve(ctx, handle, dA, dB0, dB, reps: int = 2) -> float:
    lib = ctx.lib

    def once():
        dB.copy_from(dB0, ctx.stream)
        _lib.check(lib.gblu_batch_solve(ctx.handle, handle, dA.ptr, dB.ptr, _lib.GBLU_DEVICE, None),
                   ctx.handle)

    once()
    e0, e1 = Event(), Event()
    e0.record(ctx.stream)
    for _ in range(reps):
        once()
    e1.record(ctx.stream)
    e1.synchronize()
    return e0.elapsed_ms(e1) / reps


def tune(ctx, sizes, precision: str = "fp32", A=None, b=None, use_cache: bool = True,
         budget_s: float = 60.0, sm_count: int | None = None) -> dict:
    """Search bucket edges x (threads, panel) per bucket x CTAs per bucket by
    coordinate descent on the measured solve time; returns the schedule."""
    sizes = np.ascontiguousarray(sizes, dtype=np.int64)
    sig = signature(sizes, precision)
    cache = _load_cache() if use_cache else {}
    if use_cache and sig in cache:
        return cache[sig]
    lib = ctx.lib
    if A is None or b is None:
        rng = np.random.default_rng(0)
        A = np.concatenate([(np.eye(int(n)) - 0.1 * rng.standard_normal((n, n)) / np.sqrt(n)).ravel("F")
                            for n in sizes])
        b = rng.standard_normal(int(sizes.sum()))
    dA = DeviceMatrix.from_host(np.asarray(A).reshape(-1, 1))
    dB0 = DeviceMatrix.from_host(np.asarray(b).reshape(-1, 1))
    dB = DeviceMatrix(dB0.rows, 1)
    h = ctypes.c_void_p()
    _lib.check(lib.gblu_batch_create(ctx.handle, len(sizes), sizes.ctypes.data, PRECISIONS[precision],
                                     ctypes.byref(h)), ctx.handle)
    if sm_count is None:
        sm_count = 152
    t_start = time.perf_counter()
    trials = []

    def measure(s):
        apply(ctx, h, s)
        ms = _time_solve(ctx, h, dA, dB0, dB)
        trials.append({"schedule": s, "ms": ms})
        return ms

    best, best_ms = None, float("inf")
    for edges in EDGE_SETS:
        if time.perf_counter() - t_start > budget_s:
            break
        nb = len(edges)
        cur = {"upper": list(edges), "threads": [256] * nb, "panel": [16] * nb, "ctas": [0] * nb}
        for i, hi in enumerate(edges):  # a sensible start: narrow kernels for small systems
            if hi <= 64:
                cur["threads"][i], cur["panel"][i] = 128, 8
        ms = measure(cur)
        for i in range(nb):  # coordinate descent over each bucket's variant and CTA count
            for (t, p) in VARIANTS:
                if (t, p) == (cur["threads"][i], cur["panel"][i]):
                    continue
                cand = json.loads(json.dumps(cur))
                cand["threads"][i], cand["panel"][i] = t, p
                m = measure(cand)
                if m < ms:
                    cur, ms = cand, m
            for mult in (1, 2, 4):
                cand = json.loads(json.dumps(cur))
                cand["ctas"][i] = sm_count * mult
                m = measure(cand)
                if m < ms:
                    cur, ms = cand, m
        if ms < best_ms:
            best, best_ms = cur, ms
    lib.gblu_batch_destroy(ctx.handle, h)
    dA.free(); dB0.free(); dB.free()
    result = dict(best)
    result.update({"ms": best_ms, "signature": sig, "precision": precision, "count": int(len(sizes)),
                   "trials": len(trials)})
    if use_cache:
        cache[sig] = result
        _store_cache(cache)
    return result
