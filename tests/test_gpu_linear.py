"""The LinearProblem / init / solve! interface on the GPU (the reference's
test/Core/basictests.jl:64-91 test_interface, resolve.jl, lu_refactorization.jl,
batch.jl assertions, restated)."""
import numpy as np
import pytest

from conftest import EPS64

pytestmark = pytest.mark.gpu


@pytest.fixture(params=["plain", "mixed_ir", "mixed_gmres"])
def alg(request, pkg):
    if request.param == "plain":
        return pkg.GB300LUFactorization()
    if request.param == "mixed_ir":
        return pkg.GB300MixedLUFactorization(refine="ir")
    return pkg.GB300MixedLUFactorization(refine="gmres_ir")


def test_known_answer_resolve(pkg, golden, alg):
    # test/Core/resolve.jl:78-106
    prob = pkg.LinearProblem(golden["known_A"], golden["known_b"])
    cache = pkg.init(prob, alg, alias=pkg.LinearAliasSpecifier(alias_A=False, alias_b=False))
    np.testing.assert_allclose(pkg.solve_bang(cache).u, golden["known_x"], rtol=1e-12)
    assert not cache.isfresh
    np.testing.assert_allclose(pkg.solve_bang(cache).u, golden["known_x"], rtol=1e-12)


def test_interface_A_then_b(pkg, oracle_mod, alg):
    # test/Core/basictests.jl:64-91: solve, cache.A = A2, cache.b = b2
    rng = np.random.default_rng(21)
    n = 80
    A1 = rng.random((n, n)) + n * np.eye(n)
    A2 = rng.random((n, n)) + n * np.eye(n)
    b1, b2 = rng.random(n), rng.random(n)
    cache = pkg.init(pkg.LinearProblem(A1, b1), alg)
    sol = pkg.solve_bang(cache)
    assert pkg.successful_retcode(sol)
    assert oracle_mod.backward_error(A1, sol.u, b1) <= 10 * n * EPS64
    cache.A = A2
    assert cache.isfresh
    sol = pkg.solve_bang(cache)
    assert oracle_mod.backward_error(A2, sol.u, b1) <= 10 * n * EPS64
    cache.b = b2
    assert not cache.isfresh
    sol = pkg.solve_bang(cache)
    assert oracle_mod.backward_error(A2, sol.u, b2) <= 10 * n * EPS64


def test_b_only_resolve_skips_getrf(pkg):
    rng = np.random.default_rng(22)
    n = 64
    A = rng.standard_normal((n, n)) + n * np.eye(n)
    cache = pkg.init(pkg.LinearProblem(A, rng.random(n)), pkg.GB300LUFactorization())
    pkg.solve_bang(cache)
    calls = []
    orig = cache.cacheval.getrf
    cache.cacheval.getrf = lambda *a, **k: calls.append(1) or orig(*a, **k)
    for _ in range(3):
        cache.b = rng.random(n)
        pkg.solve_bang(cache)
    assert calls == []
    cache.A = A * 2.0
    pkg.solve_bang(cache)
    assert calls == [1]


def test_singular_failure_and_recovery(pkg, golden, alg):
    # test/Core/lu_refactorization.jl:83-110
    cache = pkg.init(pkg.LinearProblem(golden["sing_Agood"].copy(), np.ones(8)), alg,
                     alias=pkg.LinearAliasSpecifier(alias_A=True))
    assert pkg.solve_bang(cache).retcode == pkg.ReturnCode.Success
    cache.A = golden["sing_A"].copy()
    sol = pkg.solve_bang(cache)
    assert sol.retcode == pkg.ReturnCode.Failure
    assert cache.isfresh  # not reset on failure
    cache.A = golden["sing_Agood"].copy()
    sol = pkg.solve_bang(cache)
    assert sol.retcode == pkg.ReturnCode.Success
    np.testing.assert_allclose(sol.u, np.linalg.solve(golden["sing_Agood"], np.ones(8)), rtol=1e-12)


def test_multi_rhs(pkg, oracle_mod, alg):
    # test/Core/batch.jl:9-57: matrix RHS
    rng = np.random.default_rng(23)
    n, k = 12, 4
    A = rng.random((n, n)) + n * np.eye(n)
    B = rng.random((n, k))
    sol = pkg.solve(pkg.LinearProblem(A, B), alg)
    assert pkg.successful_retcode(sol)
    assert sol.u.shape == (n, k)
    np.testing.assert_allclose(sol.u, np.linalg.solve(A, B), rtol=1e-12)


def test_residual_safety(pkg):
    rng = np.random.default_rng(24)
    n = 12
    A = rng.random((n, n)) + n * np.eye(n)
    B = rng.random((n, 3))
    sol = pkg.solve(pkg.LinearProblem(A, B), pkg.GB300LUFactorization(residualsafety=True))
    assert pkg.successful_retcode(sol)
    assert sol.stats["residual_norm"] <= sol.stats["residual_tol"]


@pytest.mark.parametrize("mk", [lambda pkg: pkg.GB300LUFactorization(residualsafety=True),
                                lambda pkg: pkg.GB300MixedLUFactorization(residualsafety=True)])
def test_residual_safety_failure_only_after_refactor(pkg, mk):
    """_check_residual_safety (src/factorization.jl:127-156): with abstol =
    reltol = 0 any nonzero residual fails the check, as
    APosterioriSafetyFailure; the check runs only on solves that refactored
    (check_safety = residualsafety && isfresh)."""
    rng = np.random.default_rng(27)
    n = 200
    A = rng.standard_normal((n, n)) + 2 * np.sqrt(n) * np.eye(n)
    b = rng.standard_normal(n)
    cache = pkg.init(pkg.LinearProblem(A, b), mk(pkg), abstol=0.0, reltol=0.0)
    sol = pkg.solve_bang(cache)
    assert sol.retcode == pkg.ReturnCode.APosterioriSafetyFailure
    res = np.linalg.norm(A @ sol.u - b)
    assert res > 0 and sol.stats["residual_norm"] > 0
    cache.b = rng.standard_normal(n)  # no refactorization: no check
    assert pkg.solve_bang(cache).retcode == pkg.ReturnCode.Success
    cache.A = A.copy()  # refactorization: checked again
    assert pkg.solve_bang(cache).retcode == pkg.ReturnCode.APosterioriSafetyFailure


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("where", ["host", "device"])
def test_residual_norm_on_device(ctx, pkg, prec, where):
    """The device residual ||B - A X||_F and ||B||_F against numpy, for a
    perturbed X (residual well above rounding level), N and T."""
    rng = np.random.default_rng(28)
    n, k = 333, 3
    A = rng.standard_normal((n, n)) + 2 * np.sqrt(n) * np.eye(n)
    B = rng.standard_normal((n, k))
    X = np.asfortranarray(rng.standard_normal((n, k)) * 1e-3)
    f = ctx.factor(n, n, prec)
    f.keep_matrix(True)
    assert f.getrf(A) == 0
    for trans, M in (("N", A), ("T", A.T)):
        if where == "device":
            dX, dB = pkg.DeviceMatrix.from_host(X), pkg.DeviceMatrix.from_host(B)
            r, bn = f.residual_norm(dX, dB, trans=trans)
            dX.free(); dB.free()
        else:
            r, bn = f.residual_norm(X, B, trans=trans)
        assert abs(r - np.linalg.norm(B - M @ X)) <= 1e-12 * r
        assert abs(bn - np.linalg.norm(B)) <= 1e-13 * bn
    f.close()


def test_residual_norm_needs_kept_matrix(ctx, pkg):
    n = 64
    A, B = pkg.workloads.plain(n, 1, seed=3)
    f = ctx.factor(n, n, "fp64")
    f.getrf(A)
    with pytest.raises(pkg.GBLUError):
        f.residual_norm(B, B)
    f.close()


@pytest.mark.parametrize("n,nrhs", [(8, 1), (8, 3), (40, 1), (40, 3)])
def test_rflu_dropin(pkg, oracle_mod, n, nrhs):
    """RFLUFactorization multi-RHS and cache reuse (test/Core/basictests.jl
    "RFLUFactorization multi-RHS") with GB300RFLUFactorization swapped in; the
    cacheval unpacks as RFLU's (LU, ipiv)."""
    rng = np.random.default_rng(7 + n + nrhs)
    Ar = rng.random((n, n)) + n * np.eye(n)
    Br = rng.random((n, nrhs))
    alg = pkg.GB300RFLUFactorization()
    sol = pkg.solve(pkg.LinearProblem(Ar.copy(), Br.copy()), alg)
    np.testing.assert_allclose(sol.u, np.linalg.solve(Ar, Br), rtol=1e-12)
    cache = pkg.init(pkg.LinearProblem(Ar.copy(), Br.copy()), alg)
    np.testing.assert_allclose(pkg.solve_bang(cache).u, np.linalg.solve(Ar, Br), rtol=1e-12)
    fact, ipiv = cache.cacheval
    LU, ipiv_ref, _ = oracle_mod.getrf(Ar)
    assert np.array_equal(ipiv, ipiv_ref) and np.array_equal(fact.factors(), LU)
    A2 = Ar + np.eye(n)
    cache.A = A2.copy()
    np.testing.assert_allclose(pkg.solve_bang(cache).u, np.linalg.solve(A2, Br), rtol=1e-12)


def test_rflu_pivot_false_is_refused(pkg):
    with pytest.raises(ValueError):
        pkg.GB300RFLUFactorization(pivot=False)


def test_device_resident_inputs(pkg, oracle_mod):
    rng = np.random.default_rng(25)
    n = 300
    A = rng.standard_normal((n, n))
    b = rng.standard_normal((n, 2))
    dA = pkg.DeviceMatrix.from_host(A)
    db = pkg.DeviceMatrix.from_host(b)
    sol = pkg.solve(pkg.LinearProblem(dA, db), pkg.GB300LUFactorization())
    u = sol.u.to_host()
    LU, ipiv, _ = oracle_mod.getrf(A)
    assert np.array_equal(u, oracle_mod.getrs(LU, ipiv, b))


def test_adjoint_solve_reuses_factors(pkg, oracle_mod, alg):
    # solve!(cache; adjoint = true) (src/common.jl:1012-1027): A^T u = b with
    # the cached factorization; A is factored once
    rng = np.random.default_rng(26)
    n = 150
    A = rng.standard_normal((n, n)) + 2 * np.sqrt(n) * np.eye(n)
    b = rng.standard_normal(n)
    cache = pkg.init(pkg.LinearProblem(A, b), alg)
    calls = []
    orig = cache.cacheval.getrf
    cache.cacheval.getrf = lambda *a, **k: calls.append(1) or orig(*a, **k)
    sol = pkg.solve_bang(cache, adjoint=True)  # fresh A: factor, then the transposed solve
    assert pkg.successful_retcode(sol)
    assert oracle_mod.backward_error(A.T, sol.u, b) <= 10 * n * EPS64
    sol2 = pkg.solve_bang(cache)  # the plain solve on the same factors
    assert oracle_mod.backward_error(A, sol2.u, b) <= 10 * n * EPS64
    sol3 = pkg.solve_bang(cache, adjoint=True)
    assert oracle_mod.backward_error(A.T, sol3.u, b) <= 10 * n * EPS64
    assert len(calls) == 1
    if isinstance(alg, pkg.GB300LUFactorization):
        LU, ipiv, _ = oracle_mod.getrf(A)
        assert np.array_equal(sol3.u, oracle_mod.getrs(LU, ipiv, b, trans="T"))


def test_default_algorithm(pkg, oracle_mod):
    # init(prob) without an algorithm: defaultalg picks the GB300 LU
    # (IllConditioned, the reference's default condition) or the mixed LU
    # (WellConditioned); both reach the FP64 bound
    rng = np.random.default_rng(27)
    n = 200
    A = rng.standard_normal((n, n)) + 2 * np.sqrt(n) * np.eye(n)
    b = rng.standard_normal(n)
    cache = pkg.init(pkg.LinearProblem(A, b))
    assert isinstance(cache.alg, pkg.GB300LUFactorization)
    sol = pkg.solve_bang(cache)
    LU, ipiv, _ = oracle_mod.getrf(A)
    assert np.array_equal(sol.u, oracle_mod.getrs(LU, ipiv, b))
    well = pkg.OperatorAssumptions(True, pkg.OperatorCondition.WellConditioned)
    sol = pkg.solve(pkg.LinearProblem(A, b), assumptions=well)
    assert isinstance(sol.cache.alg, pkg.GB300MixedLUFactorization)
    assert oracle_mod.backward_error(A, sol.u, b) <= 10 * n * EPS64


def test_default_safety_fallback_reports_failure(pkg):
    # a matrix whose LU "succeeds" with non-finite results: the default
    # solver's safety check (src/default.jl:946-967) turns it into a Failure
    n = 4
    A = np.eye(n)
    A[1, 1] = 1e-310  # subnormal pivot: 1/pivot overflows to inf
    b = np.ones(n)
    sol = pkg.solve(pkg.LinearProblem(A, b))
    assert sol.retcode == pkg.ReturnCode.Failure


def test_mixed_rbt_through_the_interface(pkg, oracle_mod):
    """GB300MixedLUFactorization(pivot="rbt") through init / solve!: the
    factor is created with the butterfly transform; A then b changes keep
    the FP64 bound."""
    n = 512
    A, B = pkg.workloads.shifted(n, 2, seed=77)
    alg = pkg.GB300MixedLUFactorization(factor="bf16", pivot="rbt")
    cache = pkg.init(pkg.LinearProblem(A, B[:, 0].copy()), alg)
    sol = pkg.solve_bang(cache)
    assert sol.retcode == pkg.ReturnCode.Success
    assert oracle_mod.backward_error(A, sol.u, B[:, 0]) <= 10 * n * EPS64
    assert cache.cacheval.pivoting == "rbt"
    cache.b = B[:, 1].copy()
    sol = pkg.solve_bang(cache)
    assert oracle_mod.backward_error(A, sol.u, B[:, 1]) <= 10 * n * EPS64
