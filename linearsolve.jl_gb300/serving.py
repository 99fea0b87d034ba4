"""Python driver of the serving loop (gblu_serve_*): request submission,
completion polling, and a Poisson-arrival load generator that reports p50/p99
latency and solves/s."""
from __future__ import annotations

import ctypes
import threading
import time

import numpy as np

from . import _lib
from ._lib import check

PRECISIONS = {"fp64": _lib.GBLU_FP64, "fp32": _lib.GBLU_FP32, "bf16": _lib.GBLU_BF16,
              "fp16": _lib.GBLU_FP16}


class Server:
    def __init__(self, ctx, workers: int = 4, precision: str = "fp32", refine: str = "ir",
                 hbm_budget_bytes: int = 120 << 30, max_rhs_batch: int = 8, small_n: int = 256,
                 solve: str = "fast", max_small_batch: int = 1024, max_large: int | None = None,
                 large_n: int | None = None, pivot: str = "partial"):
        self.ctx, self.lib = ctx, ctx.lib
        cfg = _lib.ServeConfig()
        check(self.lib.gblu_serve_config_default(ctypes.byref(cfg)), None)
        cfg.workers = workers
        cfg.precision = PRECISIONS[precision]
        cfg.refine_mode = _lib.GBLU_REFINE_GMRES if refine == "gmres_ir" else _lib.GBLU_REFINE_IR
        cfg.hbm_budget_bytes = hbm_budget_bytes
        cfg.max_rhs_batch = max_rhs_batch
        cfg.small_n = small_n
        cfg.solve_mode = _lib.GBLU_SOLVE_FAST if solve == "fast" else _lib.GBLU_SOLVE_EXACT
        cfg.max_small_batch = max_small_batch
        if max_large is not None:  # large factorizations running at once (0: no limit)
            cfg.max_large = max_large
        if large_n is not None:
            cfg.large_n = large_n
        # pivoting of the mixed-precision factors: partial, tournament or rbt
        cfg.pivoting = {"partial": _lib.GBLU_PIVOT_PARTIAL, "tournament": _lib.GBLU_PIVOT_TOURNAMENT,
                        "rbt": _lib.GBLU_PIVOT_RBT}[pivot]
        h = ctypes.c_void_p()
        check(self.lib.gblu_serve_create(ctx.handle, ctypes.byref(cfg), ctypes.byref(h)), ctx.handle)
        self.h = h
        self._keep = {}  # tag -> buffers kept alive until completion

    def submit(self, tag: int, key: int, b: np.ndarray, A: np.ndarray | None = None) -> np.ndarray:
        n = b.shape[0]
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.empty(n, dtype=np.float64)
        Af = None if A is None else np.asfortranarray(A, dtype=np.float64)
        r = _lib.Request(key=key, n=n, A=None if Af is None else Af.ctypes.data, b=b.ctypes.data,
                         x=x.ctypes.data, tag=tag)
        self._keep[tag] = (Af, b, x)
        st = self.lib.gblu_serve_submit(self.h, ctypes.byref(r))
        if st != 0:
            del self._keep[tag]
            raise _lib.GBLUError(st, "gblu_serve_submit failed")
        return x

    def poll(self, max_n: int = 256, wait_ms: int = 0):
        buf = (_lib.Completion * max_n)()
        got = ctypes.c_int32()
        check(self.lib.gblu_serve_poll(self.h, buf, max_n, ctypes.byref(got), wait_ms), None)
        out = []
        for i in range(got.value):
            c = buf[i]
            d = {k: getattr(c, k) for k, _ in _lib.Completion._fields_}
            kept = self._keep.pop(c.tag, None)
            d["x"] = kept[2] if kept else None
            out.append(d)
        return out

    def stats(self) -> dict:
        s = _lib.ServeStats()
        check(self.lib.gblu_serve_get_stats(self.h, ctypes.byref(s)), None)
        return {k: getattr(s, k) for k, _ in _lib.ServeStats._fields_}

    def close(self):
        if self.h:
            self.lib.gblu_serve_destroy(self.h)
            self.h = None


GBLU_ENOTFACTORED = 5
ONE_OFF_KEY = 1 << 62  # keys of resent requests: ONE_OFF_KEY + request index


def run_stream(server: Server, requests, rate_hz: float, seed: int = 0, timeout_s: float = 300.0,
               resubmit_missing: bool = False):
    """Submit `requests` (list of dicts: key, b, A or None; with
    resubmit_missing also Aeff, the key's current matrix) with Poisson
    arrivals at `rate_hz`; return completions and the wall time.

    resubmit_missing: a solve-only request whose key's factorization was
    evicted completes with GBLU_ENOTFACTORED; the client sends it again with
    the matrix it was meant for (a factor + solve) under a one-off key
    (ONE_OFF_KEY + its index), never under its own key: requests of that key
    sent later may already carry a newer matrix, which the resent one must
    not replace.  The completion then carries "resubmitted": 1 and
    "client_latency_us", the time from the first submission to the final
    completion."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_hz, size=len(requests)) if rate_hz > 0 else np.zeros(len(requests))
    done = []
    finished = threading.Event()
    t_first = {}
    lock = threading.Lock()

    def collector():
        while len(done) < len(requests):
            got = server.poll(256, wait_ms=20)
            now = time.perf_counter()
            for d in got:
                i = d["tag"]
                if (resubmit_missing and d["status"] == GBLU_ENOTFACTORED and requests[i].get("A") is None
                        and not d.get("resubmitted")):
                    rq = requests[i]
                    server.submit(i, ONE_OFF_KEY + i, rq["b"], rq["Aeff"])
                    with lock:
                        t_first.setdefault(("resub", i), True)
                    continue
                with lock:
                    d["resubmitted"] = 1 if ("resub", i) in t_first else 0
                    d["client_latency_us"] = (now - t_first[i]) * 1e6 if i in t_first else None
                done.append(d)
        finished.set()

    th = threading.Thread(target=collector, daemon=True)
    t0 = time.perf_counter()
    th.start()
    t_next = t0
    for i, rq in enumerate(requests):
        t_next += gaps[i]
        now = time.perf_counter()
        if t_next > now:
            time.sleep(t_next - now)
        with lock:
            t_first[i] = time.perf_counter()
        server.submit(i, rq["key"], rq["b"], rq.get("A"))
    finished.wait(timeout_s)
    wall = time.perf_counter() - t0
    return done, wall


def latency_summary(done, wall: float) -> dict:
    lat = np.array([d["latency_us"] for d in done if d["status"] == 0]) / 1000.0
    ok = int((np.array([d["status"] for d in done]) == 0).sum()) if done else 0
    out = {
        "completed": ok, "failed": len(done) - ok,
        "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
        "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
        "mean_ms": float(lat.mean()) if len(lat) else None,
        "solves_per_s": ok / wall if wall > 0 else None,
        "wall_s": wall,
    }
    cl = np.array([d["client_latency_us"] for d in done
                   if d["status"] == 0 and d.get("client_latency_us") is not None]) / 1000.0
    if len(cl):
        out.update({"client_p50_ms": float(np.percentile(cl, 50)), "client_p99_ms": float(np.percentile(cl, 99)),
                    "resubmitted": int(sum(d.get("resubmitted", 0) for d in done))})
    return out
