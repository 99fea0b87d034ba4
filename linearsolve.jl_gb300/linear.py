"""LinearSolve.jl's problem / cache / solve interface over the GB300 library.

This mirrors, name for name, the part of LinearSolve.jl's public interface
that the dense LU path sits behind, so that a caller (and the tests) read
like the reference:

    prob  = LinearProblem(A, b)                     # SciMLBase.LinearProblem
    cache = init(prob, GB300LUFactorization())      # src/common.jl:700-931
    sol   = solve_bang(cache)                       # solve!(cache), common.jl:1012-1017
    solve_bang(cache, adjoint=True)                 # A^T u = b, same factors (:1012-1027)
    cache.b = b2;  solve_bang(cache)                # getrs only   (common.jl:351-353)
    cache.A = A2;  solve_bang(cache)                # refactor     (common.jl:330-348)
    sol   = solve(prob, alg)                        # common.jl:988-993

The algorithm types follow the plugin contract of
docs/src/advanced/algorithm_interface.md: refactor only when ``isfresh``
and then clear it; write into ``cache.u``; a failed factorization is a
``ReturnCode.Failure`` retcode (not an exception) and leaves ``isfresh``
set (src/factorization.jl:16-28, :716-722).
"""
from __future__ import annotations

import enum
import math
from dataclasses import dataclass, field
from typing import Any, Optional

import numpy as np

from ._cuda import DeviceMatrix
from .device import default_context


class ReturnCode(enum.Enum):
    """The SciMLBase retcodes the LU path produces."""
    Default = "Default"
    Success = "Success"
    Failure = "Failure"
    APosterioriSafetyFailure = "APosterioriSafetyFailure"


def successful_retcode(rc: "ReturnCode | LinearSolution") -> bool:
    if isinstance(rc, LinearSolution):
        rc = rc.retcode
    return rc == ReturnCode.Success


@dataclass
class LinearAliasSpecifier:
    """Aliasing of init (src/common.jl:818-842): dense defaults are no alias."""
    alias_A: Optional[bool] = None
    alias_b: Optional[bool] = None


@dataclass
class LinearProblem:
    """SciMLBase.LinearProblem(A, b; u0, p)."""
    A: Any
    b: Any
    u0: Any = None
    p: Any = None


@dataclass
class LinearSolution:
    """SciMLBase.LinearSolution fields used by the LU path."""
    u: Any
    resid: Any
    alg: Any
    retcode: ReturnCode
    iters: int = 0
    cache: Any = None
    stats: dict = field(default_factory=dict)


# ---------------------------------------------------------------------------
# Algorithms (SciMLLinearSolveAlgorithm subtypes in the Julia binding)

class AbstractDenseFactorization:
    """src/LinearSolve.jl:211.  needs_concrete_A = true; needs_square_A = true."""

    needs_concrete_A = True
    needs_square_A = True
    default_alias_A = False
    default_alias_b = False
    precision = "fp64"
    residualsafety = False
    solve = "exact"

    def factor_precision(self) -> str:
        return self.precision


class GB300LUFactorization(AbstractDenseFactorization):
    """Plain FP64 partial-pivot LU on the GB300: getrf + getrs in FP64.

    The drop-in for LUFactorization (src/factorization.jl:306-311) /
    CudaOffloadLUFactorization (src/extension_algs.jl:344-356).  Factors and
    ipiv are bit-identical to the reference's blocked LU
    (src/blocked_lufact.jl), and the solve to its back-solve
    (src/factorization.jl:433-457).

    solve: "exact" (that back-solve order, bit for bit) or "fast" (the 64 x 64
    diagonal blocks of L and U inverted once per factorization and applied as
    matrix-vector products: a shorter critical path, backward-error accurate
    but not bit-identical)."""

    def __init__(self, residualsafety: bool = False, solve: str = "exact", device: int = 0):
        if solve not in ("exact", "fast"):
            raise ValueError("solve must be 'exact' or 'fast'")
        self.residualsafety = bool(residualsafety)
        self.solve = solve
        self.device = int(device)

    def __repr__(self):
        return f"GB300LUFactorization(residualsafety={self.residualsafety})"


class GB300RFLUFactorization(GB300LUFactorization):
    """The drop-in for RFLUFactorization(; pivot = Val(true), thread =
    Val(true)) (src/extension_algs.jl:524-537, solve! in
    ext/LinearSolveRecursiveFactorizationExt.jl:15-42): the same recursive,
    partial-pivot FP64 LU (RecursiveFactorization's lu! is recursive; so is
    this library's getrf) and the same forward / back substitution, on the
    GB300.  Its cacheval has RFLU's (LU, ipiv) shape.

    pivot: True (RecursiveFactorization's Val(true)); the pivot-free
           Val(false) variant is not provided (ValueError).  On matrices whose
           column maxima sit on the diagonal (the diagonally dominant ones the
           reference tests with) the two factorizations coincide.
    thread: accepted and ignored (the GPU is the thread pool)."""

    def __init__(self, pivot: bool = True, thread: bool = True, residualsafety: bool = False,
                 device: int = 0):
        if not bool(pivot):
            raise ValueError("GB300RFLUFactorization: pivot=False (RecursiveFactorization's pivot-free "
                             "lu!) is not provided; partial pivoting only")
        super().__init__(residualsafety=residualsafety, device=device)
        self.pivot = True
        self.thread = bool(thread)

    def __repr__(self):
        return f"GB300RFLUFactorization(pivot=True, thread={self.thread}, residualsafety={self.residualsafety})"


class RFLUCacheval:
    """RFLUFactorization's cacheval shape, (LU, ipiv) (src/factorization.jl:
    232-255): unpacks as (factorization, ipiv) with ipiv the 1-based int64
    pivots of the last getrf; every other attribute is the device-resident
    factorization's."""

    def __init__(self, fact):
        object.__setattr__(self, "fact", fact)

    def _pair(self):
        return (self.fact, self.fact.ipiv())

    def __iter__(self):
        return iter(self._pair())

    def __len__(self):
        return 2

    def __getitem__(self, i):
        return self._pair()[i]

    def __getattr__(self, name):
        return getattr(object.__getattribute__(self, "fact"), name)


class GB300MixedLUFactorization(AbstractDenseFactorization):
    """Mixed precision: FP32 LU, FP64 accuracy by refinement.

    factor:  "fp32"           FP32 LU (SIMT FP32 trailing updates)
             "bf16" | "fp16"  FP32 LU whose trailing updates run on the tensor
                              cores (tcgen05) with 16-bit operands
    refine:  "ir" | "gmres_ir" (classic IR, or GMRES-IR preconditioned by the LU)
    maxiters, tol: outer refinement limits (tol None: n * eps64)
    fallback: FP64 LU when refinement stalls, or at once when the pivot
              growth of the low-precision factors exceeds growth_limit
              (None: 1 / u of the factorization's arithmetic)
    residualsafety: the a-posteriori residual check of the reference
              (src/factorization.jl:127-156), run on the device.
    solve:    the low-precision correction solve, "fast" (default) or "exact"
              (see GB300LUFactorization); refinement makes either FP64-accurate.
    pivot:    pivoting of the low-precision LU: "partial" (default), "tournament"
              or "rbt" (no pivoting after a random butterfly transform of both
              sides, n >= 4; the growth check and FP64 fallback guard it).

    Unlike the reference's CUDAOffload32MixedLUFactorization
    (ext/LinearSolveCUDAExt.jl:211-242) the result is FP64-accurate."""

    def __init__(self, factor: str = "fp32", refine: str = "ir", maxiters: int = 30,
                 tol: Optional[float] = None, fallback: bool = True, gmres_restart: int = 30,
                 gmres_tol: float = 1e-10, growth_limit: Optional[float] = None,
                 residualsafety: bool = False, solve: str = "fast", pivot: str = "partial",
                 device: int = 0):
        if factor not in ("fp32", "bf16", "fp16"):
            raise ValueError(f"unsupported factor precision {factor!r}")
        if refine not in ("ir", "gmres_ir"):
            raise ValueError("refine must be 'ir' or 'gmres_ir'")
        if solve not in ("exact", "fast"):
            raise ValueError("solve must be 'exact' or 'fast'")
        if pivot not in ("partial", "tournament", "rbt"):
            raise ValueError("pivot must be 'partial', 'tournament' or 'rbt'")
        self.solve = solve
        self.pivot = pivot
        self.precision = factor
        self.refine = refine
        self.maxiters = int(maxiters)
        self.tol = tol
        self.fallback = bool(fallback)
        self.gmres_restart = int(gmres_restart)
        self.gmres_tol = float(gmres_tol)
        self.growth_limit = growth_limit
        self.residualsafety = bool(residualsafety)
        self.device = int(device)

    def __repr__(self):
        return f"GB300MixedLUFactorization(factor={self.precision!r}, refine={self.refine!r})"


# ---------------------------------------------------------------------------
# Default algorithm choice (src/default.jl)

class OperatorCondition(enum.Enum):
    """SciMLOperators' condition hint used by the default chooser."""
    IllConditioned = "IllConditioned"
    VeryIllConditioned = "VeryIllConditioned"
    SuperIllConditioned = "SuperIllConditioned"
    WellConditioned = "WellConditioned"


@dataclass
class OperatorAssumptions:
    """OperatorAssumptions(issq; condition) (src/common.jl); the reference's
    default condition is IllConditioned."""
    issq: Optional[bool] = None
    condition: OperatorCondition = OperatorCondition.IllConditioned


class DefaultAlgorithmChoice(enum.Enum):
    """The members of DefaultAlgorithmChoice this library adds
    (src/LinearSolve.jl:330-357 lists the reference's)."""
    GB300LUFactorization = "GB300LUFactorization"
    GB300MixedLUFactorization = "GB300MixedLUFactorization"


class DefaultLinearSolver:
    """DefaultLinearSolver(alg; safetyfallback) (src/default.jl).  Resolved to
    a concrete algorithm by init; see defaultalg."""

    def __init__(self, alg: DefaultAlgorithmChoice = DefaultAlgorithmChoice.GB300LUFactorization,
                 safetyfallback: bool = True, device: int = 0):
        self.alg = DefaultAlgorithmChoice(alg)
        self.safetyfallback = bool(safetyfallback)
        self.device = int(device)

    def concrete(self):
        if self.alg == DefaultAlgorithmChoice.GB300MixedLUFactorization:
            return GB300MixedLUFactorization(factor="fp32", refine="ir", fallback=True, device=self.device)
        return GB300LUFactorization(device=self.device)

    def __repr__(self):
        return f"DefaultLinearSolver({self.alg.name}, safetyfallback={self.safetyfallback})"


def defaultalg(A, b, assump: Optional[OperatorAssumptions] = None) -> DefaultLinearSolver:
    """The dense square branch of defaultalg (src/default.jl:411-520) and its
    GPU-array branch (:277-284), with the GB300 algorithms registered:

    * square, WellConditioned      -> GB300MixedLUFactorization (FP32 LU + FP64
      refinement, falling back to the FP64 LU when refinement stalls: the
      result is FP64-accurate either way);
    * square, IllConditioned        -> GB300LUFactorization (the reference's
      default condition; plain FP64 LU as LUFactorization);
    * VeryIllConditioned / SuperIllConditioned / non-square -> the reference
      picks QR / SVD / normal equations, which this library does not provide:
      NotImplementedError."""
    m, n = _shape(A)
    assump = assump or OperatorAssumptions(issq=(m == n))
    issq = (m == n) if assump.issq is None else bool(assump.issq)
    if not issq:
        raise NotImplementedError("non-square A: the reference chooses QR / normal equations, "
                                  "which are outside this library (dense LU only)")
    if assump.condition == OperatorCondition.WellConditioned:
        return DefaultLinearSolver(DefaultAlgorithmChoice.GB300MixedLUFactorization)
    if assump.condition == OperatorCondition.IllConditioned:
        return DefaultLinearSolver(DefaultAlgorithmChoice.GB300LUFactorization)
    raise NotImplementedError(f"{assump.condition.name}: the reference chooses QR / SVD, "
                              "which are outside this library (dense LU only)")


# ---------------------------------------------------------------------------
# Cache

def _shape(x):
    return (x.rows, x.cols) if isinstance(x, DeviceMatrix) else np.shape(x)


class LinearCache:
    """src/common.jl:281-306 with the setproperty! freshness logic of :313-360."""

    _tracked = ("A", "b")

    def __init__(self, A, b, u, alg, abstol, reltol, verbose, alias_A, alias_b, context):
        object.__setattr__(self, "isfresh", True)
        object.__setattr__(self, "_ctx", context)
        object.__setattr__(self, "cacheval", None)
        object.__setattr__(self, "alg", alg)
        object.__setattr__(self, "abstol", abstol)
        object.__setattr__(self, "reltol", reltol)
        object.__setattr__(self, "verbose", verbose)
        object.__setattr__(self, "alias_A", alias_A)
        object.__setattr__(self, "alias_b", alias_b)
        object.__setattr__(self, "A", A)
        object.__setattr__(self, "b", b)
        object.__setattr__(self, "u", u)
        object.__setattr__(self, "stats", {})
        object.__setattr__(self, "default", None)  # the DefaultLinearSolver init resolved, if any

    def __setattr__(self, name, value):
        if name == "A":
            # cache.A = X  =>  isfresh = true (common.jl:330-348)
            if not isinstance(value, DeviceMatrix):
                value = np.asarray(value)
            object.__setattr__(self, "A", value)
            object.__setattr__(self, "isfresh", True)
        elif name == "b":
            # cache.b = y  =>  no refactorization (common.jl:351-353)
            if not isinstance(value, DeviceMatrix):
                value = np.asarray(value)
            object.__setattr__(self, "b", value)
        else:
            object.__setattr__(self, name, value)


def _default_tolerances(A):
    dt = np.float64
    eps = float(np.finfo(dt).eps)
    return math.sqrt(eps), math.sqrt(eps)  # abstol, reltol defaults of common.jl


def init(prob: LinearProblem, alg=None, alias: Optional[LinearAliasSpecifier] = None,
         abstol: Optional[float] = None, reltol: Optional[float] = None, verbose: bool = False,
         context=None, assumptions: Optional[OperatorAssumptions] = None) -> LinearCache:
    """SciMLBase.init(prob, alg; alias, abstol, reltol, verbose, assumptions)
    (common.jl:700-931).  alg None picks defaultalg(A, b, assumptions)."""
    default = None
    if alg is None:
        alg = defaultalg(prob.A, prob.b, assumptions)
    if isinstance(alg, DefaultLinearSolver):
        default, alg = alg, alg.concrete()
    A, b = prob.A, prob.b
    m, n = _shape(A)
    if getattr(alg, "needs_square_A", False) and m != n:
        raise ValueError(f"{type(alg).__name__} requires a square A, got {m}x{n}")
    if _shape(b)[0] != m:
        raise ValueError("b has the wrong number of rows")
    alias = alias or LinearAliasSpecifier()
    alias_A = alg.default_alias_A if alias.alias_A is None else bool(alias.alias_A)
    alias_b = alg.default_alias_b if alias.alias_b is None else bool(alias.alias_b)
    if not isinstance(A, DeviceMatrix):
        A = np.asarray(A, dtype=np.float64)
        if not alias_A:
            A = np.array(A, order="F", copy=True)
    if not isinstance(b, DeviceMatrix):
        b = np.asarray(b, dtype=np.float64)
        if not alias_b:
            b = np.array(b, copy=True)
    if prob.u0 is not None:
        u = np.array(prob.u0, dtype=np.float64, copy=True)
    elif isinstance(b, DeviceMatrix):
        u = DeviceMatrix(b.rows, b.cols)
    else:
        u = np.zeros(np.shape(b), dtype=np.float64)
    d_abs, d_rel = _default_tolerances(A)
    ctx = context if context is not None else default_context(getattr(alg, "device", 0))
    cache = LinearCache(A, b, u, alg, d_abs if abstol is None else abstol,
                        d_rel if reltol is None else reltol, verbose, alias_A, alias_b, ctx)
    # init_cacheval: the device-resident factorization object, allocated once
    fact = ctx.factor(m, n, alg.factor_precision())
    if m == n:
        fact.set_solve(alg.solve)
    if isinstance(alg, GB300MixedLUFactorization) and alg.pivot != "partial":
        fact.set_pivoting(alg.pivot)
    if alg.residualsafety:
        fact.keep_matrix(True)  # the FP64 copy of A the residual check reads (A_backup)
    cache.cacheval = RFLUCacheval(fact) if isinstance(alg, GB300RFLUFactorization) else fact
    cache.default = default
    return cache


def _solve_into(cache: LinearCache, fact, b, trans: str = "N"):
    alg = cache.alg
    if isinstance(alg, GB300MixedLUFactorization):
        if isinstance(b, DeviceMatrix):
            out = cache.u if isinstance(cache.u, DeviceMatrix) else DeviceMatrix(b.rows, b.cols)
            out.copy_from(b)
            from ._cuda import device_synchronize
            device_synchronize()
            X, stats = fact.solve_refined(out, trans=trans, mode=alg.refine, max_iter=alg.maxiters,
                                          tol=alg.tol or 0.0, fallback=alg.fallback,
                                          gmres_restart=alg.gmres_restart, gmres_tol=alg.gmres_tol,
                                          growth_limit=alg.growth_limit or 0.0)
            return out, stats
        X, stats = fact.solve_refined(b, trans=trans, mode=alg.refine, max_iter=alg.maxiters,
                                      tol=alg.tol or 0.0, fallback=alg.fallback,
                                      gmres_restart=alg.gmres_restart, gmres_tol=alg.gmres_tol,
                                      growth_limit=alg.growth_limit or 0.0)
        return X, stats
    if isinstance(b, DeviceMatrix):
        out = cache.u if isinstance(cache.u, DeviceMatrix) else DeviceMatrix(b.rows, b.cols)
        out.copy_from(b)
        from ._cuda import device_synchronize
        device_synchronize()
        fact.getrs(out, trans=trans)
        return out, {}
    return fact.getrs(b, trans=trans), {}


def _store_u(cache: LinearCache, u):
    if isinstance(u, DeviceMatrix):
        cache.u = u
    elif isinstance(cache.u, np.ndarray) and cache.u.shape == np.shape(u):
        cache.u[...] = u
    else:
        cache.u = np.array(u)


def _finite(u) -> bool:
    return bool(np.all(np.isfinite(u.to_host() if isinstance(u, DeviceMatrix) else u)))


def solve_bang(cache: LinearCache, adjoint: bool = False, **kwargs) -> LinearSolution:
    """solve!(cache; adjoint) (common.jl:1012-1027).

    adjoint=True solves A^T u = b with the cached factors (the reuse of
    _solve_adjoint!, src/adjoint_factorization.jl): getrs / the refined solve
    with trans 'T', factoring first only when A is fresh."""
    if adjoint:
        if cache.isfresh:
            sol = _solve_bang(cache)
            if sol.retcode == ReturnCode.Failure:
                return sol
        u, stats = _solve_into(cache, cache.cacheval, cache.b, trans="T")
        _store_u(cache, u)
        cache.stats = stats
        return LinearSolution(cache.u, None, cache.alg, ReturnCode.Success,
                              iters=stats.get("iterations", 0), cache=cache, stats=stats)
    sol = _solve_bang(cache)
    default = getattr(cache, "default", None)
    if default is not None and default.safetyfallback and sol.retcode == ReturnCode.Success \
            and not _finite(sol.u):
        # _default_lu_solve_with_fallback (src/default.jl:946-967) retries with
        # QR, which this library does not provide: report the failure instead
        sol.retcode = ReturnCode.Failure
        sol.stats = dict(sol.stats, fallback="non-finite LU solution; QR is outside this library")
    return sol


def _solve_bang(cache: LinearCache) -> LinearSolution:
    """solve!(cache, alg) for the GB300 algorithms (factorization.jl:643-736 shape)."""
    alg = cache.alg
    fact = cache.cacheval
    # the reference checks the residual after the solves that refactored
    # (check_safety = alg.residualsafety && cache.isfresh, factorization.jl:647)
    check_safety = bool(getattr(alg, "residualsafety", False)) and cache.isfresh
    if cache.isfresh:
        A_now = cache.A
        info = fact.getrf(A_now)
        if info != 0:
            # Failure without resetting isfresh (factorization.jl:16-28, :716-722)
            if cache.verbose:
                print("Solver failed")
            return LinearSolution(cache.u, None, alg, ReturnCode.Failure, cache=cache,
                                  stats={"info": info})
        cache.isfresh = False
    u, stats = _solve_into(cache, fact, cache.b)
    _store_u(cache, u)
    cache.stats = stats
    if check_safety:
        # _check_residual_safety (factorization.jl:127-156): ||A u - b|| against
        # abstol + reltol ||b||, 2-norms as the reference, computed on the
        # device from the FP64 A the factorization kept
        res, bnorm = fact.residual_norm(cache.u, cache.b)
        tol = cache.abstol + cache.reltol * bnorm
        stats = dict(stats, residual_norm=res, residual_tol=tol)
        cache.stats = stats
        if res > tol:
            return LinearSolution(cache.u, None, alg, ReturnCode.APosterioriSafetyFailure,
                                  cache=cache, stats=stats)
    return LinearSolution(cache.u, None, alg, ReturnCode.Success, iters=stats.get("iterations", 0),
                          cache=cache, stats=stats)


def solve(prob: LinearProblem, alg=None, adjoint: bool = False, **kwargs) -> LinearSolution:
    """solve(prob, alg; kwargs...) = solve!(init(prob, alg; kwargs...)) (common.jl:988-993)."""
    return solve_bang(init(prob, alg, **kwargs), adjoint=adjoint)


def reinit(cache: LinearCache, A=None, b=None) -> LinearCache:
    """reinit!(cache; A, b) funnels into the same setters (common.jl:933-964)."""
    if A is not None:
        cache.A = A
    if b is not None:
        cache.b = b
    return cache
