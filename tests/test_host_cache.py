"""The host side of the LinearSolve mirror (linear.py) on the CPU: when a
cache refactors, what it writes, how failures are reported, aliasing, the
residual-safety branch, adjoint solves, and what init asks of the factor
object.  The device factor is replaced by a recording stand-in built on
scipy's LAPACK (test infrastructure only), so every branch of the host logic
runs without a GPU; the same behaviour on the device is covered by
test_gpu_linear.py.

The conventions checked are the reference's: setproperty! on
LinearCache (src/common.jl:313-360: cache.A = X marks the cache fresh,
cache.b = y does not), solve! refactoring only when fresh
(src/factorization.jl:643-736), a zero pivot reported as
ReturnCode.Failure without clearing isfresh (:16-28, :716-722), dense
algorithms copying A and b at init by default (src/common.jl:818-842), and
_check_residual_safety after refactoring solves only (:127-156)."""
import numpy as np
import pytest
from scipy.linalg import lapack


class _Factor:
    """Records the calls the host logic makes; computes with LAPACK."""

    def __init__(self, log, m, n, precision):
        self.log, self.m, self.n, self.precision = log, m, n, precision
        self.lu = self.piv = None
        self.A = None
        self.residual = None  # forced residual norm for the safety branch
        log.append(("create", m, n, precision))

    def set_solve(self, mode):
        self.log.append(("set_solve", mode))

    def set_pivoting(self, mode):
        self.log.append(("set_pivoting", mode))

    def keep_matrix(self, keep):
        self.log.append(("keep_matrix", keep))

    def getrf(self, A):
        self.log.append(("getrf",))
        self.A = np.array(A, dtype=np.float64)
        self.lu, self.piv, info = lapack.dgetrf(self.A)
        return int(info)

    def getrs(self, B, trans="N"):
        self.log.append(("getrs", trans))
        X, info = lapack.dgetrs(self.lu, self.piv, np.array(B, dtype=np.float64),
                                trans=0 if trans == "N" else 1)
        assert info == 0
        return X

    def solve_refined(self, B, trans="N", **kw):
        self.log.append(("solve_refined", trans, kw["mode"]))
        return self.getrs(B, trans), {"iterations": 2, "fell_back": 0}

    def residual_norm(self, u, b):
        self.log.append(("residual_norm",))
        r = self.A @ np.asarray(u) - np.asarray(b)
        res = float(np.linalg.norm(r)) if self.residual is None else self.residual
        return res, float(np.linalg.norm(b))

    def ipiv(self):
        return self.piv.astype(np.int64) + 1

    def factors(self):
        return self.lu


class _Context:
    def __init__(self):
        self.log = []
        self.made = []

    def factor(self, m, n, precision="fp64"):
        f = _Factor(self.log, m, n, precision)
        self.made.append(f)
        return f


def _problem(pkg, n=12, seed=0):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, n)) + n * np.eye(n)
    b = rng.standard_normal(n)
    return pkg.LinearProblem(A, b), A, b


def _count(log, name):
    return sum(1 for e in log if e[0] == name)


def test_refactors_only_when_fresh(pkg):
    prob, A, b = _problem(pkg)
    ctx = _Context()
    cache = pkg.init(prob, pkg.GB300LUFactorization(), context=ctx)
    assert cache.isfresh
    u_obj = cache.u
    sol = pkg.solve_bang(cache)
    assert sol.retcode == pkg.ReturnCode.Success and not cache.isfresh
    assert np.allclose(A @ sol.u, b)
    assert cache.u is u_obj  # written into cache.u
    assert (_count(ctx.log, "getrf"), _count(ctx.log, "getrs")) == (1, 1)
    b2 = b[::-1].copy()
    cache.b = b2  # new b: back-substitution only
    assert not cache.isfresh
    sol = pkg.solve_bang(cache)
    assert np.allclose(A @ sol.u, b2)
    assert (_count(ctx.log, "getrf"), _count(ctx.log, "getrs")) == (1, 2)
    A2 = A + np.eye(A.shape[0])
    cache.A = A2  # new A: fresh, refactored on the next solve
    assert cache.isfresh
    sol = pkg.solve_bang(cache)
    assert np.allclose(A2 @ sol.u, b2)
    assert (_count(ctx.log, "getrf"), _count(ctx.log, "getrs")) == (2, 3)
    pkg.reinit(cache, b=b)  # reinit! funnels into the same setters
    assert not cache.isfresh
    pkg.reinit(cache, A=A)
    assert cache.isfresh
    assert _count(ctx.log, "create") == 1  # one factor object for the cache's life


def test_zero_pivot_is_a_failure_retcode(pkg):
    n = 6
    A = np.eye(n)
    A[:, 3] = 0.0  # exact zero pivot in column 4
    ctx = _Context()
    cache = pkg.init(pkg.LinearProblem(A, np.ones(n)), pkg.GB300LUFactorization(), context=ctx)
    sol = pkg.solve_bang(cache)
    assert sol.retcode == pkg.ReturnCode.Failure
    assert sol.stats["info"] == 4
    assert not pkg.successful_retcode(sol)
    assert cache.isfresh  # not cleared: the next solve factors again
    assert _count(ctx.log, "getrs") == 0
    cache.A = np.eye(n) * 2.0
    sol = pkg.solve_bang(cache)
    assert sol.retcode == pkg.ReturnCode.Success and np.allclose(sol.u, 0.5)


@pytest.mark.parametrize("alias_A,alias_b", [(None, None), (True, True), (False, True)])
def test_alias_semantics(pkg, alias_A, alias_b):
    prob, A, b = _problem(pkg, seed=1)
    A0, b0 = A.copy(), b.copy()
    spec = pkg.LinearAliasSpecifier(alias_A=alias_A, alias_b=alias_b)
    cache = pkg.init(prob, pkg.GB300LUFactorization(), alias=spec, context=_Context())
    A[0, 0] += 100.0
    b[0] += 100.0
    # dense default: no alias (copies at init)
    assert np.array_equal(cache.A, A if alias_A else A0)
    assert np.array_equal(cache.b, b if alias_b else b0)


def test_residual_safety_checked_after_refactoring_only(pkg):
    prob, A, b = _problem(pkg, seed=2)
    ctx = _Context()
    cache = pkg.init(prob, pkg.GB300LUFactorization(residualsafety=True), context=ctx)
    assert ("keep_matrix", True) in ctx.log  # the FP64 A the check reads stays on the device
    sol = pkg.solve_bang(cache)
    assert sol.retcode == pkg.ReturnCode.Success
    assert sol.stats["residual_norm"] <= sol.stats["residual_tol"]
    assert _count(ctx.log, "residual_norm") == 1
    cache.b = b * 2.0
    pkg.solve_bang(cache)  # not fresh: no check (check_safety = residualsafety && isfresh)
    assert _count(ctx.log, "residual_norm") == 1
    ctx.made[0].residual = 1e3  # a residual above abstol + reltol ||b||
    cache.A = A
    sol = pkg.solve_bang(cache)
    assert sol.retcode == pkg.ReturnCode.APosterioriSafetyFailure
    assert not pkg.successful_retcode(sol)


def test_adjoint_reuses_the_factors(pkg):
    prob, A, b = _problem(pkg, seed=3)
    ctx = _Context()
    cache = pkg.init(prob, pkg.GB300LUFactorization(), context=ctx)
    sol = pkg.solve_bang(cache, adjoint=True)  # fresh: factor first, then the 'T' solve
    assert np.allclose(A.T @ sol.u, b)
    assert _count(ctx.log, "getrf") == 1 and ("getrs", "T") in ctx.log
    sol = pkg.solve_bang(cache)
    assert np.allclose(A @ sol.u, b)
    assert _count(ctx.log, "getrf") == 1  # the same factors serve both


@pytest.mark.parametrize("pivot", ["partial", "rbt", "tournament"])
def test_mixed_init_configures_the_factor(pkg, pivot):
    prob, A, b = _problem(pkg, seed=4)
    ctx = _Context()
    alg = pkg.GB300MixedLUFactorization(factor="bf16", refine="gmres_ir", pivot=pivot)
    cache = pkg.init(prob, alg, context=ctx)
    assert ctx.log[0] == ("create", 12, 12, "bf16")
    assert ("set_solve", "fast") in ctx.log
    # partial pivoting is the factor's default: set only when another is asked for
    assert (("set_pivoting", pivot) in ctx.log) == (pivot != "partial")
    sol = pkg.solve_bang(cache)
    assert sol.retcode == pkg.ReturnCode.Success and sol.iters == 2
    assert ("solve_refined", "N", "gmres_ir") in ctx.log
    assert np.allclose(A @ sol.u, b)


def test_rflu_cacheval_has_the_reference_shape(pkg):
    prob, A, b = _problem(pkg, seed=5)
    cache = pkg.init(prob, pkg.GB300RFLUFactorization(), context=_Context())
    pkg.solve_bang(cache)
    fact, ipiv = cache.cacheval  # RFLU's (LU, ipiv)
    assert len(cache.cacheval) == 2 and ipiv.dtype == np.int64
    P = np.eye(12)
    for k, p in enumerate(ipiv - 1):  # LAPACK interchange sequence, 1-based
        P[[k, p]] = P[[p, k]]
    L = np.tril(fact.factors(), -1) + np.eye(12)
    U = np.triu(fact.factors())
    assert np.allclose(P @ A, L @ U)


def test_needs_square_and_matching_b(pkg):
    with pytest.raises(ValueError):
        pkg.init(pkg.LinearProblem(np.zeros((4, 3)), np.zeros(4)), pkg.GB300LUFactorization(),
                 context=_Context())
    with pytest.raises(ValueError):
        pkg.init(pkg.LinearProblem(np.eye(4), np.zeros(5)), pkg.GB300LUFactorization(),
                 context=_Context())
