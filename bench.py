#!/usr/bin/env python
"""Benchmark: FP64-accurate solves/s of the dense LU path on GB300.

Workload (one step): plain FP64 LU of an n = 8192 matrix (A iid N(0,1)) and
16 successive single right-hand-side solves through that one cached
factorization (1 getrf + 16 getrs), the cached-LinearCache pattern of
solve!(cache) / cache.b = b.  Inputs are seeded synthetic arrays.

  value  solves/s with A and B resident in HBM (device-timed, CUDA events on
         the library's stream)
  e2e    the same step through the public interface (LinearProblem / init /
         solve!) with pinned host buffers: the H2D copy of A and of each b and
         the D2H copy of each solution are inside the timed region.

--impl reference times the CPU implementation of the same path (LAPACK
dgetrf/dgetrs on OpenBLAS, the routines LinearSolve.jl's LUFactorization calls)
on the host cores.

--suite adds sub-objects to the line (comma list, or "all"; by default all of
them on one GPU, about three minutes, and none on several; --suite '' for
none):
  config1     n = 1000, A and b iid N(0,1) (seed 0), 1 RHS: GPU getrf + getrs
              (device-resident and through solve!) beside CPU LAPACK
  mixed       n = 16384, A = G + 4 sqrt(n) I, 4 RHS: FP32/BF16/FP16 LU + FP64
              refinement vs the plain FP64 LU, both to the FP64 bound
  mixed_hard  n = 16384, A = Q1 diag(s) Q2^T, s log-spaced 1..1e6, 4 RHS: FP32
              LU + FP64 GMRES-IR (and plain IR) vs the plain FP64 LU
  batched     20,000 uneven systems n in [8, 256]: FP64 and FP32 + FP64 IR
  serving     Poisson stream, n log-uniform in [64, 4096], p50/p99 latency
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

EPS64 = float(np.finfo(np.float64).eps)
# FP64 roofline denominator.  MEASURED_PEAKS.json has no FP64 figure (tcgen05
# has no FP64 kind, so FP64 runs on the FP64 pipe); the bench measures it on
# the GPU it runs on with a DFMA probe (libgblu_tools.so: 16 independent
# register-operand FMA chains per thread, swept launch shapes, event-timed)
# and reports NVIDIA's published GB300 FP64 rate beside it.
FP64_NOMINAL_TFLOPS = 1.25
METRIC = "FP64-accurate solves/s (1 getrf + 16 cached getrs, n=8192, plain FP64 LU)"
UNIT = "solves/s"


def headline_config(n: int, nrhs: int, world: int) -> dict:
    """The workload both arms (--impl gblu and --impl reference) print."""
    return {"workload": f"plain FP64 LU n={n}, 1 getrf + {nrhs} cached single-RHS getrs per step",
            "n": n, "nrhs": nrhs, "seed": 0, "global_batch": nrhs * world,
            "l2": ("inputs larger than L2 (A = %.0f MB, L2 129 MB)" if 8 * n * n > 129e6
                   else "inputs fit in L2 (A = %.0f MB, L2 129 MB)") % (8 * n * n / 1e6)}


def fp64_peak(probe):
    """(peak TFLOP/s, source) of the FP64 roofline: the probe when it ran."""
    if probe and probe.get("tflops"):
        return probe["tflops"], ("DFMA probe on this GPU (%.3f TFLOP/s, %s); nominal GB300 FP64 %.2f"
                                 % (probe["tflops"], probe["shape"], FP64_NOMINAL_TFLOPS))
    return FP64_NOMINAL_TFLOPS, "nominal GB300 FP64 %.2f TFLOP/s (probe unavailable)" % FP64_NOMINAL_TFLOPS


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


class Dist:
    """Barrier and max-over-ranks for N > 1 (gloo: host-side plumbing only)."""

    def __init__(self, world: int):
        self.world = world
        self.pg = None
        if world > 1:
            import torch.distributed as td
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def peak_fp64_probe(device: int):
    """FP64 FMA rate measured on this GPU, with the SM clocks seen meanwhile."""
    import ctypes
    path = os.path.join(ROOT, "linearsolve.jl_gb300", "libgblu_tools.so")
    lib = ctypes.CDLL(path)
    fn = lib.gblu_tool_peak_fp64_shape
    fn.argtypes = [ctypes.c_int32, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int32)]
    fn.restype = ctypes.c_int32
    out = ctypes.c_double()
    shape = (ctypes.c_int32 * 2)()
    clocks = ClockSampler(device)
    clocks.start()
    st = fn(device, ctypes.byref(out), shape)
    clk = clocks.stop()
    if st != 0:
        return None
    return {"tflops": float(out.value), "shape": f"{shape[0]} CTAs/SM x {shape[1]} threads",
            "sm_mhz": clk.get("sm_mhz"), "reasons": clk.get("reasons")}


def cpu_model() -> str:
    """Host CPU model and core count, for the CPU baseline's label."""
    model = ""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                model = ln.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return f"{model or platform.processor() or 'unknown'} ({platform.machine()}, {os.cpu_count()} cores)"


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def profile_traffic(kind: str):
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as fh:
            return json.load(fh).get(kind)
    except (OSError, ValueError):
        return None


# ---------------------------------------------------------------------------
# CPU reference arm

def cpu_lapack_steps(A, B, steps: int, want_x: bool = False):
    """LAPACK getrf + one getrs per RHS column (the cached-solve pattern);
    with want_x also the solutions of the last step."""
    import oracle
    times = []
    X = None
    for _ in range(steps):
        t0 = time.perf_counter()
        LU, ipiv, info = oracle.lapack_getrf(A)
        cols = [oracle.lapack_getrs(LU, ipiv, B[:, j:j + 1]) for j in range(B.shape[1])]
        times.append(time.perf_counter() - t0)
        if want_x:
            X = np.concatenate([np.asarray(c).reshape(-1, 1) for c in cols], axis=1)
    return (times, X) if want_x else times


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    import oracle  # noqa: F401  (CPU implementation of the path; not the product)
    pkg = load_pkg()
    n, nrhs = args.n, args.nrhs
    A, B = pkg.workloads.plain(n, nrhs, seed=0)
    cpu_lapack_steps(A, B, args.warmup)
    times = cpu_lapack_steps(A, B, args.steps)
    total = sum(times)
    value = args.steps * nrhs / total
    cores = os.cpu_count()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded N(0,1), numpy default_rng(0))",
        "impl": "reference", "parallelism": f"host threads x{cores}", "cpu_model": cpu_model(),
        "config": headline_config(n, nrhs, world),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{args.steps} full steps: scipy.linalg.lapack dgetrf + {nrhs} dgetrs "
                                   f"(OpenBLAS, all {cores} host threads) -- the LAPACK routines "
                                   "LUFactorization reaches through LinearAlgebra.lu!/ldiv!"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# GPU arm

def load_pkg():
    import __graft_entry__ as ge
    return ge.load_package()


def run_gpu(args, rank, world, local):
    dist = Dist(world)
    pkg = load_pkg()
    from importlib import import_module
    cu = import_module(pkg.__name__ + "._cuda")
    n, nrhs = args.n, args.nrhs
    ctx = pkg.Context(local)
    stream = ctx.stream
    if args.only_suite:  # profiling aid: the suite parts alone, one JSON object
        if args.suite == "auto":
            args.suite = ",".join(SUITES)
        args.peak_fp64, args.peak_fp64_source = fp64_peak(None)
        out = run_suites(pkg, cu, ctx, args)
        if rank == 0:
            print(json.dumps(out))
        dist.close()
        return 0
    A, B = pkg.workloads.plain(n, nrhs, seed=0)

    # ---- device-resident workload (value) ----
    dA = pkg.DeviceMatrix.from_host(A)
    dB0 = pkg.DeviceMatrix.from_host(B)
    dB = pkg.DeviceMatrix(n, nrhs)
    f = ctx.factor(n, n, "fp64")
    cols = [cu.DeviceColumn(dB, j) for j in range(nrhs)]

    def step():
        dB.copy_from(dB0, stream)
        info = f.getrf(dA)
        if info != 0:
            raise RuntimeError(f"getrf info={info}")
        for c in cols:
            f.getrs(c)

    for _ in range(args.warmup):
        step()
    cu.device_synchronize()
    # accuracy of the last step (not timed)
    X = dB.to_host()
    berr = max(pkg_backward_error(A, X[:, j], B[:, j]) for j in range(nrhs))

    # timed region: the library's own launch path (getrf replayed from the
    # factor's captured graph, no per-launch events); the counters still count
    # every launch, graph replays included
    clocks = ClockSampler(local)
    clocks.start()
    ctx.profile_enable(False)  # resets the counters
    dist.barrier()
    cu.device_synchronize()
    e0, e1 = cu.Event(), cu.Event()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    e1.synchronize()
    cu.device_synchronize()
    dist.barrier()
    launches = ctx.profile_read(reset=True)["launches"]
    clk = clocks.stop()
    t_ms = dist.max(e0.elapsed_ms(e1))
    total_solves = dist.sum(args.steps * nrhs)
    value = total_solves / (t_ms / 1000.0)

    # the same steps again with per-launch events on the library's stream:
    # per-kernel device time and the roofline of the dominant kernel
    ctx.profile_enable(True)
    p0, p1 = cu.Event(), cu.Event()
    p0.record(stream)
    for _ in range(args.steps):
        step()
    p1.record(stream)
    p1.synchronize()
    prof = ctx.profile_read(reset=True)
    ctx.profile_enable(False)
    profiled_ms = p0.elapsed_ms(p1) / args.steps

    # ---- the same step with the fast getrs (inverted diagonal blocks) ----
    fast = None
    if rank == 0:
        ff = ctx.factor(n, n, "fp64")
        ff.set_solve("fast")
        dBf = pkg.DeviceMatrix(n, nrhs)
        colsf = [cu.DeviceColumn(dBf, j) for j in range(nrhs)]

        def step_fast():
            dBf.copy_from(dB0, stream)
            ff.getrf(dA)
            for c in colsf:
                ff.getrs(c)

        for _ in range(max(3, args.warmup)):
            step_fast()
        f0, f1 = cu.Event(), cu.Event()
        f0.record(stream)
        for _ in range(args.steps):
            step_fast()
        f1.record(stream)
        f1.synchronize()
        ms_fast = f0.elapsed_ms(f1) / args.steps
        ctx.profile_enable(True)
        step_fast()
        pf = ctx.profile_read(reset=True)
        ctx.profile_enable(False)
        Xf = dBf.to_host()
        fast = {"solve": "fast (64 x 64 diagonal blocks of L and U inverted after getrf)",
                "value": nrhs / (ms_fast / 1e3), "unit": UNIT, "ms_per_step": ms_fast,
                "getrs_ms_per_solve": pf["getrs"]["ms"] / nrhs,
                "backward_error": max(pkg_backward_error(A, Xf[:, j], B[:, j]) for j in range(nrhs)),
                "forward_error_vs_exact": _forward_error(Xf, X)}
        dBf.free()
        ff.close()

    # ---- end to end through the public interface, pinned host buffers ----
    pA = cu.PinnedArray((n, n))
    pA.array[...] = A
    pB = cu.PinnedArray((n, nrhs))
    pB.array[...] = B
    alg = pkg.GB300LUFactorization()
    cache = pkg.init(pkg.LinearProblem(pA.array, pB.array[:, 0]), alg,
                     alias=pkg.LinearAliasSpecifier(alias_A=True, alias_b=True), context=ctx)

    def e2e_step():
        cache.A = pA.array
        for j in range(nrhs):
            cache.b = pB.array[:, j]
            sol = pkg.solve_bang(cache)
            if sol.retcode != pkg.ReturnCode.Success:
                raise RuntimeError("e2e solve failed")

    for _ in range(max(1, args.warmup)):
        e2e_step()
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    t_e2e = dist.max(time.perf_counter() - t0)
    e2e_value = dist.sum(args.steps * nrhs) / t_e2e

    # ---- roofline of the dominant kernel (event-timed over the profiled steps) ----
    kinds = [k for k in prof if k != "launches"]
    dom = max(kinds, key=lambda k: prof[k]["ms"])
    d = prof[dom]
    peaks = measured_peaks()
    probe = peak_fp64_probe(local) if rank == 0 else None
    peak_fp64, peak_src = fp64_peak(probe)
    args.peak_fp64, args.peak_fp64_source = peak_fp64, peak_src
    if dom in ("gemm", "panel", "trsm"):
        achieved = d["flops"] / (d["ms"] / 1000.0) / 1e12 if d["ms"] > 0 else 0.0
        roof = {"bound": "fp64 pipe", "achieved": achieved, "peak": peak_fp64, "unit": "TFLOP/s",
                "frac": (achieved / peak_fp64) if peak_fp64 else None,
                "peak_source": peak_src, "fp64_probe": probe,
                "frac_of_nominal": achieved / FP64_NOMINAL_TFLOPS,
                "kernel": f"{dom} (FP64)", "launches": d["count"],
                "flops_per_launch": d["flops"] / max(d["count"], 1),
                "ms_per_launch": d["ms"] / max(d["count"], 1)}
    else:
        achieved = d["bytes"] / (d["ms"] / 1000.0) / 1e9 if d["ms"] > 0 else 0.0
        peak = peaks.get("hbm_gbs")
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": (achieved / peak) if peak else None,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs", "kernel": dom,
                "launches": d["count"]}
    roof["timed_over"] = (f"{args.steps} steps with per-launch CUDA events on the library stream "
                          f"({profiled_ms:.1f} ms/step with events vs {t_ms / args.steps:.1f} ms/step "
                          "in the timed region)")
    tr = profile_traffic(dom)
    if tr and d["count"]:
        # captured DRAM bytes scale with the algorithmic bytes of a launch
        roof["traffic"] = tr["ratio_to_algorithmic"] * d["bytes"] / d["count"]
        roof["traffic_source"] = ("ncu dram__bytes_read+write of one captured launch (%s), scaled "
                                  "per launch by algorithmic bytes" % tr["captured_launch"])
    else:
        roof["traffic"] = None

    # per-phase fractions of the roofline: getrf against the FP64 peak, getrs
    # against HBM (its algorithmic bytes: both triangles read once per solve)
    step_ms = {k: prof[k]["ms"] / args.steps for k in kinds}
    getrf_ms = sum(step_ms.get(k, 0.0) for k in ("gemm", "panel", "laswp", "trsm", "perm"))
    getrs_ms = step_ms.get("getrs", 0.0)
    hbm = peaks.get("hbm_gbs")
    getrf_tf = getrf_flops(n) / (getrf_ms / 1e3) / 1e12 if getrf_ms > 0 else None
    getrs_gbs = nrhs * (8.0 * n * n + 16.0 * n) / (getrs_ms / 1e3) / 1e9 if getrs_ms > 0 else None
    phases = {
        "getrf": {"achieved": getrf_tf, "unit": "TFLOP/s", "peak": peak_fp64,
                  "frac": getrf_tf / peak_fp64 if getrf_tf and peak_fp64 else None,
                  "bound": "fp64 pipe (" + peak_src + ")", "flops": getrf_flops(n), "ms": getrf_ms},
        "getrs": {"achieved": getrs_gbs, "unit": "GB/s", "peak": hbm,
                  "frac": getrs_gbs / hbm if getrs_gbs and hbm else None,
                  "bound": "HBM (the sweeps are latency-bound wavefronts)",
                  "bytes_per_solve": 8.0 * n * n + 16.0 * n, "ms": getrs_ms},
    }

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded N(0,1), numpy default_rng(0))",
        "parallelism": f"replicas x{world}",
        "config": headline_config(n, nrhs, world),
        "accuracy": {"backward_error": berr, "bound": 10 * n * EPS64},
        "clocks": clk,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 8 * n * n + nrhs * 8 * n,
                "d2h_bytes_per_step": nrhs * 8 * n + 8},
        "gpu_launches": launches,
        "roofline": roof,
        "roofline_by_phase": phases,
        "kernel_ms": {k: round(prof[k]["ms"] / args.steps, 3) for k in kinds if prof[k]["count"]},
    }
    if fast is not None:
        line["getrs_fast"] = fast

    if world > 1:  # the batched workload sharded over the ranks' GPUs (every rank takes part)
        sharded = run_batched_sharded(pkg, cu, ctx, args, dist, rank, world)
        if rank == 0:
            line["batched_sharded"] = sharded

    if args.suite == "auto":
        args.suite = ",".join(SUITES) if world == 1 else ""
    if args.suite and rank == 0:
        line.update(run_suites(pkg, cu, ctx, args))

    if rank == 0 and not args.no_cpu:
        # bounded CPU sample of the same workload on this host
        ts, Xl = cpu_lapack_steps(A, B, args.cpu_steps, want_x=True)
        cv = args.cpu_steps * nrhs / sum(ts)
        if Xl is not None:  # forward error of the GPU solutions against LAPACK's
            line["accuracy"]["forward_error_vs_lapack"] = float(np.abs(X - Xl).max() / np.abs(Xl).max())
        line["cpu_baseline"] = {
            "value": cv, "unit": UNIT, "cores": os.cpu_count(), "kind": "port", "cpu_model": cpu_model(),
            "sample": f"{args.cpu_steps} full steps: scipy.linalg.lapack dgetrf + {nrhs} dgetrs (OpenBLAS, "
                      f"{os.cpu_count()} host threads), the LAPACK routines LUFactorization calls"}
    if rank == 0:
        print(json.dumps(line))
    dist.close()
    return 0


def pkg_backward_error(A, x, b):
    r = b - A @ x
    nA = np.abs(A).sum(axis=1).max()
    return float(np.abs(r).max() / (nA * np.abs(x).max() + np.abs(b).max()))


def _timed_solve(pkg, cu, ctx, f, dA, dB0, dB, prec, reps, mode="ir", warm=3, **refine_kw):
    """getrf + (getrs | refined solve) from the device-resident A, timed with
    events on the context stream; returns (ms, refinement stats, kernel_ms)."""

    def once():
        dB.copy_from(dB0, ctx.stream)
        f.getrf(dA)
        if prec == "fp64":
            f.getrs(dB)
            return {}
        _, st = f.solve_refined(dB, mode=mode, **refine_kw)
        return st

    for _ in range(warm):  # warm-up; the library replays a factor's getrf from a graph from its third run
        once()
    cu.device_synchronize()
    e0, e1 = cu.Event(), cu.Event()
    e0.record(ctx.stream)
    st = {}
    for _ in range(reps):  # timed without the per-launch profiling events
        st = once()
    e1.record(ctx.stream)
    e1.synchronize()
    ms = e0.elapsed_ms(e1) / reps
    ctx.profile_enable(True)  # one more run for the per-kernel split
    once()
    prof = ctx.profile_read(reset=True)
    ctx.profile_enable(False)
    kms = {k: round(v["ms"], 3) for k, v in prof.items() if k != "launches" and v["count"]}
    return ms, st, kms


def _forward_error(X, Xref):
    return float(np.abs(X - Xref).max() / np.abs(Xref).max())


SUITES = ("config1", "mixed", "mixed_hard", "batched", "serving")


def run_suites(pkg, cu, ctx, args) -> dict:
    """The comparison suites, each in its own sub-object; a suite that fails
    records its error instead of losing the line."""
    parts = set(p for p in args.suite.split(",") if p)
    if "all" in parts:
        parts = set(SUITES)
    runners = {"config1": run_config1_suite, "mixed": run_mixed_suite,
               "mixed_hard": run_mixed_hard_suite, "batched": run_batched_suite,
               "serving": run_serving_suite}
    out = {}
    for name in SUITES:
        if name not in parts:
            continue
        t0 = time.perf_counter()
        try:
            out[name] = runners[name](pkg, cu, ctx, args)
        except Exception as e:  # noqa: BLE001 - reported in the line
            out[name] = {"error": f"{type(e).__name__}: {e}"}
        out[name]["suite_wall_s"] = round(time.perf_counter() - t0, 1)
    return out


def run_config1_suite(pkg, cu, ctx, args):
    """n = 1000, A and b iid N(0,1) from default_rng(0), one RHS (the
    reference's CPU-runnable configuration): plain FP64 getrf + getrs on the
    GPU, device-resident and end to end through init / solve! with a new A
    per solve, beside LAPACK dgetrf + dgetrs on all host cores (median of 20
    runs after 5 warm-ups)."""
    n, reps = 1000, 20
    A, B = pkg.workloads.plain(n, 1, seed=0)
    b = np.ascontiguousarray(B[:, 0])
    dA = pkg.DeviceMatrix.from_host(A)
    dB0 = pkg.DeviceMatrix.from_host(B)
    dB = pkg.DeviceMatrix(n, 1)
    f = ctx.factor(n, n, "fp64")
    ms, _, kms = _timed_solve(pkg, cu, ctx, f, dA, dB0, dB, "fp64", reps)
    X = dB.to_host()[:, 0]
    f.close()
    dA.free(); dB0.free(); dB.free()
    alg = pkg.GB300LUFactorization()
    cache = pkg.init(pkg.LinearProblem(A.copy(order="F"), b.copy()), alg, context=ctx)

    def e2e_once():
        cache.A = A
        cache.b = b
        sol = pkg.solve_bang(cache)
        if sol.retcode != pkg.ReturnCode.Success:
            raise RuntimeError("config1 solve failed")
        return sol.u

    for _ in range(3):
        e2e_once()
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        e2e_once()
        ts.append(time.perf_counter() - t0)
    e2e_ms = 1e3 * statistics.median(ts)
    import oracle
    for _ in range(5):
        oracle.lapack_solve(A, B)
    cts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        Xl, _ = oracle.lapack_solve(A, B)
        cts.append(time.perf_counter() - t0)
    cpu_ms = 1e3 * statistics.median(cts)
    Xl = np.asarray(Xl).reshape(-1)
    out = {"n": n, "nrhs": 1, "seed": 0,
           "gpu_ms_per_solve": ms, "gpu_solves_per_s": 1e3 / ms,
           "e2e_ms_per_solve": e2e_ms, "e2e_solves_per_s": 1e3 / e2e_ms,
           "e2e_path": "init/solve! with host A and b: H2D of A and b, getrf, getrs, D2H of x per solve",
           "cpu_lapack_ms_per_solve": cpu_ms, "cpu_solves_per_s": 1e3 / cpu_ms,
           "cpu": {"kind": "port", "impl": "scipy.linalg.lapack dgetrf + dgetrs (OpenBLAS)",
                   "cores": os.cpu_count(), "cpu_model": cpu_model(), "runs": reps},
           "backward_error": pkg_backward_error(A, X, b), "bound": 10 * n * EPS64,
           "forward_error_vs_lapack": _forward_error(X, Xl),
           "kernel_ms": kms,
           "getrf_roofline": getrf_phase_roofline(kms, n, "fp64", args)}
    return out


def run_mixed_suite(pkg, cu, ctx, args):
    """n = 16384, A = G + 4 sqrt(n) I, 4 RHS: FP32/BF16/FP16 LU + FP64 IR vs
    plain FP64 LU; the forward error of each is taken against the plain FP64
    solution (the reference algorithm's result, bit for bit).  Variants: the
    exact or fast correction solve, and partial pivoting or none after a
    random butterfly transform ("rbt")."""
    n, nrhs = args.mixed_n, 4
    A, B = pkg.workloads.shifted(n, nrhs, seed=1)
    dA = pkg.DeviceMatrix.from_host(A)
    dB0 = pkg.DeviceMatrix.from_host(B)
    dB = pkg.DeviceMatrix(n, nrhs)
    out = {"n": n, "nrhs": nrhs, "A": "G + 4 sqrt(n) I"}
    X64 = None
    variants = (("fp64_plain", "fp64", "exact", "partial"), ("fp32_ir", "fp32", "exact", "partial"),
                ("bf16_ir", "bf16", "exact", "partial"), ("fp16_ir", "fp16", "exact", "partial"),
                ("fp32_ir_fast_solve", "fp32", "fast", "partial"), ("bf16_ir_fast_solve", "bf16", "fast", "partial"),
                ("fp16_ir_fast_solve", "fp16", "fast", "partial"), ("fp32_rbt_ir_fast_solve", "fp32", "fast", "rbt"),
                ("bf16_rbt_ir_fast_solve", "bf16", "fast", "rbt"), ("fp16_rbt_ir_fast_solve", "fp16", "fast", "rbt"))
    for label, prec, solve, pivot in variants:
        f = ctx.factor(n, n, prec)
        f.set_solve(solve)  # the low-precision correction solve (mixed factors default to fast)
        if pivot != "partial":
            f.set_pivoting(pivot)
        # the FP64 solve set takes seconds: one warm-up and one timed run
        ms, st, kms = _timed_solve(pkg, cu, ctx, f, dA, dB0, dB, prec, 1 if prec == "fp64" else 3,
                                   warm=1 if prec == "fp64" else 3)
        X = dB.to_host()
        if X64 is None:
            X64 = X.copy()
        be = max(pkg_backward_error(A, X[:, j], B[:, j]) for j in range(nrhs))
        out[label] = {"ms_per_solve_set": ms, "solves_per_s": nrhs / (ms / 1000), "backward_error": be,
                      "forward_error_vs_fp64": _forward_error(X, X64), "stats": st, "kernel_ms": kms,
                      "getrf_roofline": getrf_phase_roofline(kms, n, prec, args)}
        f.close()
    for label, _, _, _ in variants[1:]:
        out["speedup_%s_vs_fp64" % label] = out[label]["solves_per_s"] / out["fp64_plain"]["solves_per_s"]
    out["bound"] = 10 * n * EPS64
    dA.free(); dB0.free(); dB.free()
    if not args.no_cpu:
        # the reference's CPU path on this host: LAPACK dgetrf + dgetrs (4 RHS), one
        # warm-up and two timed runs (a bounded sample: seconds per run at this n)
        import oracle
        oracle.lapack_solve(A, B)
        ts = []
        for _ in range(2):
            t0 = time.perf_counter()
            Xc, _ = oracle.lapack_solve(A, B)
            ts.append(time.perf_counter() - t0)
        cms = 1e3 * statistics.median(ts)
        out["cpu_baseline"] = {"ms_per_solve_set": cms, "solves_per_s": nrhs / (cms / 1e3), "kind": "port",
                               "impl": "scipy.linalg.lapack dgetrf + dgetrs (OpenBLAS)", "cores": os.cpu_count(),
                               "cpu_model": cpu_model(), "runs": len(ts),
                               "backward_error": max(pkg_backward_error(A, np.asarray(Xc)[:, j], B[:, j])
                                                     for j in range(nrhs))}
    return out


def run_mixed_hard_suite(pkg, cu, ctx, args):
    """n = 16384, A = Q1 diag(s) Q2^T with s log-spaced 1..1e6, 4 RHS: FP32 LU
    with FP64 GMRES-IR vs plain FP64 LU."""
    n, nrhs, cond = args.mixed_n, 4, 1e6
    t0 = time.perf_counter()
    A, B = pkg.workloads.svd_conditioned_gpu(n, nrhs, cond, seed=2)
    gen_s = time.perf_counter() - t0
    dA = pkg.DeviceMatrix.from_host(A)
    dB0 = pkg.DeviceMatrix.from_host(B)
    dB = pkg.DeviceMatrix(n, nrhs)
    out = {"n": n, "nrhs": nrhs, "A": "Q1 diag(s) Q2^T, s log-spaced 1..1e6", "input_generation_s": gen_s}
    X64 = None
    variants = (("fp64_plain", "fp64", "ir", {}),
                ("fp32_gmres_ir", "fp32", "gmres_ir", {"solve": "exact"}),
                ("fp32_gmres_ir_inner_tol_1e-6", "fp32", "gmres_ir", {"gmres_tol": 1e-6, "solve": "exact"}),
                ("fp32_ir", "fp32", "ir", {"solve": "exact"}),
                ("fp32_gmres_ir_fast_solve", "fp32", "gmres_ir", {"solve": "fast"}),
                ("fp32_gmres_ir_fast_solve_inner_tol_1e-6", "fp32", "gmres_ir", {"gmres_tol": 1e-6, "solve": "fast"}),
                ("fp32_ir_fast_solve", "fp32", "ir", {"solve": "fast"}))
    for label, prec, mode, kw in variants:
        f = ctx.factor(n, n, prec)
        kw = dict(kw)
        f.set_solve(kw.pop("solve", "exact"))  # the low-precision preconditioner solve
        pivot = kw.pop("pivot", "partial")
        if pivot != "partial":
            f.set_pivoting(pivot)
        ms, st, kms = _timed_solve(pkg, cu, ctx, f, dA, dB0, dB, prec, 1 if prec == "fp64" else 2,
                                   mode=mode, warm=1 if prec == "fp64" else 3, **kw)
        X = dB.to_host()
        if X64 is None:
            X64 = X.copy()
        be = max(pkg_backward_error(A, X[:, j], B[:, j]) for j in range(nrhs))
        out[label] = {"ms_per_solve_set": ms, "solves_per_s": nrhs / (ms / 1000), "backward_error": be,
                      "forward_error_vs_fp64": _forward_error(X, X64), "stats": st, "kernel_ms": kms}
        f.close()
    for label, _, _, _ in variants[1:]:
        out["speedup_%s_vs_fp64" % label] = out[label]["solves_per_s"] / out["fp64_plain"]["solves_per_s"]
    out["bound"] = 10 * n * EPS64
    dA.free(); dB0.free(); dB.free()
    return out


def run_batched_suite(pkg, cu, ctx, args):
    """20,000 systems, n_i ~ U{8..256}, A_i = I - g_i J_i: one graph launch per solve."""
    import ctypes
    lib = ctx.lib
    sizes, A, b, _ = pkg.workloads.batch(args.batch_count, seed=0)
    a_off, b_off = pkg.workloads.offsets(sizes)
    dA = pkg.DeviceMatrix.from_host(A.reshape(-1, 1))
    dB0 = pkg.DeviceMatrix.from_host(b.reshape(-1, 1))
    dB = pkg.DeviceMatrix(len(b), 1)
    out = {"count": int(len(sizes)), "n_range": [int(sizes.min()), int(sizes.max())],
           "a_bytes": int(A.nbytes), "lu_flops": float(sum(pkg_lu_flops(int(n)) for n in sizes))}
    for label, prec in (("fp64", 0), ("fp32_ir", 1)):
        h = ctypes.c_void_p()
        sz = np.ascontiguousarray(sizes, dtype=np.int64)
        st = lib.gblu_batch_create(ctx.handle, len(sz), sz.ctypes.data, prec, ctypes.byref(h))
        if st != 0:
            out[label] = {"error": lib.gblu_last_error(ctx.handle).decode()}
            continue
        info = np.zeros(len(sz), dtype=np.int64)

        def once():
            dB.copy_from(dB0, ctx.stream)
            st2 = lib.gblu_batch_solve(ctx.handle, h, dA.ptr, dB.ptr, 1, info.ctypes.data)
            if st2 != 0:
                raise RuntimeError(lib.gblu_last_error(ctx.handle).decode())

        once()
        e0, e1 = cu.Event(), cu.Event()
        reps = 3
        e0.record(ctx.stream)
        for _ in range(reps):
            once()
        e1.record(ctx.stream)
        e1.synchronize()
        ms = e0.elapsed_ms(e1) / reps
        X = dB.to_host()[:, 0]
        worst = 0.0
        rng = np.random.default_rng(1)
        for i in rng.choice(len(sizes), size=min(200, len(sizes)), replace=False):
            n = int(sizes[i])
            Ai = A[a_off[i]:a_off[i] + n * n].reshape(n, n, order="F")
            worst = max(worst, pkg_backward_error(Ai, X[b_off[i]:b_off[i] + n], b[b_off[i]:b_off[i] + n]) / n)
        gf = out["lu_flops"] / (ms / 1000.0) / 1e9
        out[label] = {"ms_per_batch": ms, "solves_per_s": len(sizes) / (ms / 1000.0), "gflops": gf,
                      "max_backward_error_over_n_eps": worst / EPS64,
                      "failed_info": int((info != 0).sum())}
        pk = getattr(args, "peak_fp64", None)
        if prec == 0 and pk:
            out[label]["frac_of_fp64_peak"] = gf / (pk * 1000.0)
        if prec != 0:  # refinement corrections per system; -1 = re-solved by the FP64 kernel
            its = np.zeros(len(sz), dtype=np.int32)
            if lib.gblu_batch_iterations(ctx.handle, h, its.ctypes.data) == 0:
                vals, cnts = np.unique(its, return_counts=True)
                out[label]["iterations"] = {str(int(v)): int(c) for v, c in zip(vals, cnts)}
        lib.gblu_batch_destroy(ctx.handle, h)
    out["speedup_fp32_ir_vs_fp64"] = out["fp32_ir"]["solves_per_s"] / out["fp64"]["solves_per_s"]
    # CPU: LAPACK loop over a bounded sample of the same systems, all host threads
    import oracle
    k = min(2000, len(sizes))
    t0 = time.perf_counter()
    for i in range(k):
        n = int(sizes[i])
        LU, ipiv, _ = oracle.lapack_getrf(A[a_off[i]:a_off[i] + n * n].reshape(n, n, order="F"))
        oracle.lapack_getrs(LU, ipiv, b[b_off[i]:b_off[i] + n])
    dt = time.perf_counter() - t0
    out["cpu_baseline"] = {"solves_per_s": k / dt, "sample": f"first {k} systems, scipy LAPACK loop",
                           "cores": os.cpu_count()}
    dA.free(); dB0.free(); dB.free()
    return out


def run_batched_sharded(pkg, cu, ctx, args, dist, rank, world):
    """The 20,000 uneven systems split over the N ranks (greedy balance of
    sum n^3, no exchange on the data path): each rank solves its shard with
    the batched kernels of its own GPU; timing is the max over ranks of the
    event-timed solves (strong scaling: the total work is fixed); the shards'
    solutions are gathered on rank 0 afterwards and sampled for accuracy."""
    import torch.distributed as td
    from importlib import import_module
    sh = import_module(pkg.__name__ + ".sharding")
    sizes, A, b, _ = pkg.workloads.batch(args.batch_count, seed=0)
    parts = sh.shard_systems(sizes, world)
    idx = parts[rank]
    ss, As, bs = sh.pack(sizes, A, b, idx)
    bt = pkg.Batch(ctx, ss, "fp64")
    dA = pkg.DeviceMatrix.from_host(As.reshape(-1, 1))
    dB0 = pkg.DeviceMatrix.from_host(bs.reshape(-1, 1))
    dB = pkg.DeviceMatrix(len(bs), 1)

    def once():
        dB.copy_from(dB0, ctx.stream)
        bt.solve(dA, dB)

    once()
    reps = 3
    dist.barrier()
    cu.device_synchronize()
    e0, e1 = cu.Event(), cu.Event()
    e0.record(ctx.stream)
    for _ in range(reps):
        once()
    e1.record(ctx.stream)
    e1.synchronize()
    ms = dist.max(e0.elapsed_ms(e1) / reps)
    x_sub = dB.to_host()[:, 0]
    gathered = [None] * world
    td.all_gather_object(gathered, (idx, x_sub))
    bt.close()
    dA.free(); dB0.free(); dB.free()
    if rank != 0:
        return None
    a_off, b_off = pkg.workloads.offsets(sizes)
    x = np.empty(len(b))
    for ridx, rx in gathered:
        pos = 0
        for i in ridx:
            n = int(sizes[i])
            x[b_off[i]:b_off[i] + n] = rx[pos:pos + n]
            pos += n
    worst = 0.0
    rng = np.random.default_rng(1)
    for i in rng.choice(len(sizes), size=min(200, len(sizes)), replace=False):
        n = int(sizes[i])
        Ai = A[a_off[i]:a_off[i] + n * n].reshape(n, n, order="F")
        worst = max(worst, pkg_backward_error(Ai, x[b_off[i]:b_off[i] + n], b[b_off[i]:b_off[i] + n]) / n)
    loads = [float((sizes[p].astype(float) ** 3).sum()) for p in parts]
    return {"count": int(len(sizes)), "ranks": world, "scaling": "strong (fixed 20,000 systems split over the ranks)",
            "ms_per_batch": ms, "solves_per_s": len(sizes) / (ms / 1e3), "precision": "fp64",
            "load_balance_max_over_min": max(loads) / max(min(loads), 1.0),
            "max_backward_error_over_n_eps": worst / EPS64}


def pkg_lu_flops(n):
    return 2.0 * n ** 3 / 3.0 + 2.0 * n * n


def getrf_flops(n):
    """LAPACK's operation count of a square getrf."""
    return 2.0 * n ** 3 / 3.0 - n * n / 2.0 - n / 6.0


def getrf_phase_roofline(kms, n, prec, args):
    """Fraction of the peak reached by the factorization phase of a mixed-suite
    run (its kernel split comes from one extra run with per-launch events)."""
    ms = sum(kms.get(k, 0.0) for k in ("gemm", "panel", "laswp", "trsm", "perm"))
    if ms <= 0:
        return None
    tf = getrf_flops(n) / (ms / 1e3) / 1e12
    if prec in ("bf16", "fp16"):
        peak, src = measured_peaks().get("bf16_tflops"), "MEASURED_PEAKS.json bf16_tflops (tensor, burst)"
    elif prec == "fp64":
        peak, src = getattr(args, "peak_fp64", None), getattr(args, "peak_fp64_source", "")
    else:
        return {"achieved": tf, "unit": "TFLOP/s", "ms": ms, "peak": None,
                "note": "FP32 SIMT update: no measured FP32 peak"}
    return {"achieved": tf, "unit": "TFLOP/s", "ms": ms, "peak": peak, "peak_source": src,
            "frac": tf / peak if peak else None}


def serving_workload(pkg, nkeys: int, nreq: int, seed: int = 0):
    """The served keys and stream.  Every key gets its own size, n
    log-uniform in [64, 4096] (so the keys hold hundreds of distinct sizes),
    and a first matrix (A = G + 4 sqrt(n) I, G iid N(0,1)): the warm
    requests, which fill the resident cache before the stream starts.  The
    stream itself is 30% new A and 70% new b against the key's current
    matrix.  The Gaussian parts are n x n windows at random offsets of one
    seeded 8192 x 8192 pool, so building a thousand requests is a copy."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(64), np.log(4096), size=nkeys)).astype(int)
    pool = rng.standard_normal((8192, 8192))

    def matrix(n):
        r0, c0 = (int(v) for v in rng.integers(0, 8192 - n + 1, size=2))
        A = np.asfortranarray(pool[r0:r0 + n, c0:c0 + n])
        A[np.diag_indices(n)] += 4.0 * np.sqrt(n)
        return A

    cur = {}
    warm = []
    for k in range(nkeys):
        cur[k] = matrix(int(sizes[k]))
        warm.append({"key": k, "A": cur[k], "b": rng.standard_normal(sizes[k]), "Aeff": cur[k]})
    reqs = []
    for _ in range(nreq):
        k = int(rng.integers(nkeys))
        if rng.random() < 0.3:
            cur[k] = matrix(int(sizes[k]))
            reqs.append({"key": k, "A": cur[k], "b": rng.standard_normal(sizes[k]), "Aeff": cur[k]})
        else:
            reqs.append({"key": k, "A": None, "b": rng.standard_normal(sizes[k]), "Aeff": cur[k]})
    del pool
    return sizes, warm, reqs


def run_serving_suite(pkg, cu, ctx, args):
    """Poisson stream against resident factorizations: n log-uniform in [64,
    4096], one size per key; each server first factors every key's matrix
    (the warm phase, all at once, untimed), then the timed stream is 30% new
    A and 70% new b.  Mixed FP32 factors with FP64 refinement (fast inner
    solve), systems with n <= 256 batched across keys through the batched
    kernels.  Budget 120 GB at the swept rates, and one rate with a budget
    small enough that the warm phase already evicts: admission waits and
    evictions happen, and a solve on an evicted key is sent again with its
    matrix (its client latency counts both trips).  Then the 400 Hz stream
    once more with --serve-variant's factors (default BF16 with no pivoting
    after the butterfly transform)."""
    from importlib import import_module
    serving = import_module(pkg.__name__ + ".serving")
    nkeys = args.serve_keys
    sizes, warm, reqs = serving_workload(pkg, nkeys, args.serve_requests, seed=0)
    out = {"keys": nkeys, "distinct_sizes": int(len(np.unique(sizes))), "warm_requests": len(warm),
           "requests": len(reqs), "n_range": [int(sizes.min()), int(sizes.max())],
           "new_A_fraction": float(np.mean([r["A"] is not None for r in reqs])),
           "precision": f"{args.serve_precision} factors ({args.serve_pivot} pivoting) + FP64 IR "
                        "(fast inner solve); n <= 256 on the batched lane",
           "target": "p99 <= 35 ms at 400 Hz, backward error <= 10 n eps64", "rates": []}
    base = (args.serve_precision, args.serve_pivot)
    runs = [(r, 120 << 30, base) for r in args.serve_rates] + [
        (400.0, int(args.serve_small_budget_gb * 2 ** 30), base)]
    if args.serve_variant[0] and tuple(args.serve_variant) != base:  # the same stream, other factors
        runs.append((400.0, 120 << 30, tuple(args.serve_variant)))
    for rate, budget, (precision, pivot) in runs:
        clocks = ClockSampler(ctx.device)  # the stream's GPU clocks (the tail varies with them)
        srv = serving.Server(ctx, workers=4, precision=precision, hbm_budget_bytes=budget,
                             max_large=args.serve_max_large, pivot=pivot)
        small = budget < (120 << 30)
        wdone, wwall = serving.run_stream(srv, warm, rate_hz=0.0, seed=1)
        st0 = srv.stats()
        clocks.start()
        done, wall = serving.run_stream(srv, reqs, rate_hz=rate, seed=int(rate), resubmit_missing=small)
        clk = clocks.stop()
        st = srv.stats()
        srv.close()
        summ = serving.latency_summary(done, wall)
        worst = 0.0
        for d in done:
            if d["status"] == 0 and d["tag"] % 7 == 0:
                i = d["tag"]
                n = len(reqs[i]["b"])
                worst = max(worst, pkg_backward_error(reqs[i]["Aeff"], d["x"], reqs[i]["b"]) / (n * EPS64))
        summ.update({"offered_rate_hz": rate, "budget_gb": budget / 2 ** 30, "clocks": clk,
                     "factors": f"{precision}, {pivot} pivoting",
                     "max_backward_error_over_n_eps": worst, "warm_s": wwall,
                     "warm_failed": int(sum(d["status"] != 0 for d in wdone)),
                     "merged_solves": st["merged_solves"] - st0["merged_solves"],
                     "factorizations": st["factorizations"] - st0["factorizations"],
                     "evictions": st["evictions"] - st0["evictions"],
                     "warm_evictions": st0["evictions"],
                     "admission_waits": st["admission_waits"] - st0["admission_waits"],
                     "small_launches": st["small_launches"] - st0["small_launches"],
                     "small_systems": st["small_systems"] - st0["small_systems"]})
        out["rates"].append(summ)
    return out


KERNEL_CASES = ("gemm_bf16", "gemm_fp16", "gemm_fp32", "refine", "perm", "mixed_bf16", "mixed_bf16_rbt",
                "step_fp64", "getrs_fast", "helpers")


def run_kernel_case(args) -> int:
    """One small invocation of a group of kernels, for ncu (no timing, no
    JSON line): operands larger than L2 so DRAM counters mean something.
      gemm_bf16 / gemm_fp16  C -= A B, M = N = K = 4096 through gblu_gemm_update
                             (conv_a / col_scale / conv_b + tc_gemm_kernel)
      gemm_fp32              the same on the FP32 SIMT path (gemm_sub_f32_rb_kernel)
      refine                 FP32 factor of n = 6144 (convert_f64_f32, umax) and refined
                             solves of 4 RHS, IR then GMRES-IR (gemv partial / reduce,
                             colmax, pow2_scales, scale_to_f32, update_from_f32, axpby)
      perm                   LAPACK-shaped dgetrs with host factors and pivots, n = 8192
                             (upload_ipiv_check_kernel, perm_from_ipiv_kernel)
      mixed_bf16             the mixed suite's BF16 solve set, n = 16384, 4 RHS, run twice
                             (launch lists: every kernel of getrf + refined solve)
      mixed_bf16_rbt         the same with no pivoting after the random butterfly transform
      step_fp64              two steps of the headline workload (n = 8192, 1 getrf + 16 getrs)
      getrs_fast             the same factorization, then 8 single-RHS solves in fast mode
      helpers                n = 6144: BF16 factor (trsm_inv / trsm_inv_apply, prepare and
                             its reduction, diag_inverse of the fast solve) with a GMRES-IR
                             solve (gmres_begin / step / scale / finish); the same factor
                             with tournament pivoting (tslu_select / tslu_apply); an FP64
                             factor's device residual check (sumsq_partial / final); an
                             FP64 n = 4096 factor on the shared-memory cluster panel
                             (panel_cluster_kernel, forced with GBLU_PANEL=cluster); a BF16
                             factor with no pivoting after the butterfly transform
                             (rbt_matrix, genp_panel, rbt_vec)"""
    pkg = load_pkg()
    _, _, local = dist_env()
    ctx = pkg.Context(local)
    rng = np.random.default_rng(5)
    case = args.kernel_case
    if case.startswith("gemm_"):
        m = n = k = 4096
        A = rng.uniform(-1, 1, size=(m, k)).astype(np.float32)
        B = rng.standard_normal((k, n)).astype(np.float32)
        C = rng.standard_normal((m, n)).astype(np.float32)
        for _ in range(2):
            ctx.gemm_update(C, A, B, case.split("_")[1])
    elif case == "refine":
        n = 6144
        A, B = pkg.workloads.shifted(n, 4, seed=3)
        f = ctx.factor(n, n, "fp32")
        f.getrf(A)
        f.solve_refined(B, mode="ir")
        f.solve_refined(B, mode="gmres_ir")
        f.close()
    elif case == "perm":
        n = 8192
        A, B = pkg.workloads.plain(n, 1, seed=4)
        LU, ipiv, _ = pkg.dgetrf(A)
        pkg.dgetrs(LU, ipiv, B)
    elif case in ("mixed_bf16", "mixed_bf16_rbt"):
        n = args.mixed_n
        A, B = pkg.workloads.shifted(n, 4, seed=1)
        dA = pkg.DeviceMatrix.from_host(A)
        dB = pkg.DeviceMatrix.from_host(B)
        f = ctx.factor(n, n, "bf16")
        if case == "mixed_bf16_rbt":
            f.set_pivoting("rbt")
        for _ in range(2):
            dB.copy_from(pkg.DeviceMatrix.from_host(B))
            f.getrf(dA)
            f.solve_refined(dB)
        f.close()
    elif case == "getrs_fast":
        n = args.n
        A, B = pkg.workloads.plain(n, 8, seed=0)
        dA = pkg.DeviceMatrix.from_host(A)
        f = ctx.factor(n, n, "fp64")
        f.set_solve("fast")
        f.getrf(dA)
        for j in range(8):
            f.getrs(pkg.DeviceMatrix.from_host(B[:, j:j + 1]))
        f.close()
    elif case == "helpers":
        n = 6144
        A, B = pkg.workloads.shifted(n, 4, seed=6)
        f = ctx.factor(n, n, "bf16")
        f.getrf(A)
        f.solve_refined(B, mode="gmres_ir")
        f.close()
        os.environ["GBLU_PANEL"] = "tournament"  # read when the factor is created
        f = ctx.factor(n, n, "bf16")
        del os.environ["GBLU_PANEL"]
        f.getrf(A)
        f.close()
        g = ctx.factor(n, n, "fp64")
        g.keep_matrix(True)
        g.getrf(A)
        X = g.getrs(B)
        g.residual_norm(X, B)
        g.close()
        os.environ["GBLU_PANEL"] = "cluster"  # read at each getrf
        A2, _ = pkg.workloads.plain(4096, 1, seed=7)
        g = ctx.factor(4096, 4096, "fp64")
        g.getrf(A2)
        g.close()
        del os.environ["GBLU_PANEL"]
        f = ctx.factor(n, n, "bf16")
        f.set_pivoting("rbt")
        f.getrf(A)
        f.solve_refined(B)
        f.close()
    elif case == "step_fp64":
        n, nrhs = args.n, args.nrhs
        A, B = pkg.workloads.plain(n, nrhs, seed=0)
        dA = pkg.DeviceMatrix.from_host(A)
        f = ctx.factor(n, n, "fp64")
        for _ in range(2):
            f.getrf(dA)
            for j in range(nrhs):
                f.getrs(pkg.DeviceMatrix.from_host(B[:, j:j + 1]))
        f.close()
    else:
        raise SystemExit(f"unknown kernel case {case!r}; one of {KERNEL_CASES}")
    ctx.close()
    print(f"kernel case {case} done")
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gblu", choices=["gblu", "reference"])
    ap.add_argument("--n", type=int, default=8192)
    ap.add_argument("--nrhs", type=int, default=16)
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--suite", default="auto",
                    help="comma list of config1,mixed,mixed_hard,batched,serving (or all); '' for none; "
                         "auto = all of them on one GPU; none on several (the batched workload is then "
                         "sharded across the ranks instead)")
    ap.add_argument("--batch-count", type=int, default=20000)
    ap.add_argument("--only-suite", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=1000)
    ap.add_argument("--mixed-n", type=int, default=16384)
    ap.add_argument("--serve-rates", type=float, nargs="*", default=[100.0, 400.0, 0.0])
    ap.add_argument("--serve-keys", type=int, default=300)
    ap.add_argument("--serve-small-budget-gb", type=float, default=0.5)
    ap.add_argument("--serve-max-large", type=int, default=None,
                    help="large factorizations (n >= 2048) running at once (0: no limit; default: the library's)")
    ap.add_argument("--serve-precision", choices=("fp32", "bf16", "fp16"), default="fp32",
                    help="factor precision of the serving suite's mixed factors")
    ap.add_argument("--serve-pivot", choices=("partial", "tournament", "rbt"), default="partial",
                    help="pivoting of the serving suite's mixed factors")
    ap.add_argument("--serve-variant", nargs=2, default=["bf16", "rbt"], metavar=("PRECISION", "PIVOT"),
                    help="one more 400 Hz stream with these factors ('' '' for none)")
    ap.add_argument("--kernel-case", choices=KERNEL_CASES, default=None,
                    help="run one small case of a kernel group once (for ncu) and exit")
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.kernel_case:
        return run_kernel_case(args)
    if args.impl == "reference":
        return run_reference(args, rank, world)
    return run_gpu(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
