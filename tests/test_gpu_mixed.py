"""Mixed precision: FP32 factors + FP64 refinement reach the FP64 backward
error bound; stalls fall back to the FP64 LU."""
import numpy as np
import pytest

from conftest import EPS64

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", ["ir", "gmres_ir"])
@pytest.mark.parametrize("n,nrhs", [(64, 1), (500, 4), (2048, 4)])
def test_shifted_reaches_fp64(ctx, oracle_mod, pkg, mode, n, nrhs):
    A, B = pkg.workloads.shifted(n, nrhs, seed=n)
    f = ctx.factor(n, n, "fp32")
    assert f.getrf(A) == 0
    X, st = f.solve_refined(B, mode=mode)
    be = oracle_mod.backward_error(A, X, B)
    assert be <= 10 * n * EPS64, (be, st)
    assert st["converged"] == 1 and st["fell_back"] == 0
    Xl, _ = oracle_mod.lapack_solve(A, B)
    assert oracle_mod.forward_error(X, Xl) < 1e-10
    f.close()


@pytest.mark.parametrize("mode", ["ir", "gmres_ir"])
def test_ill_conditioned(ctx, oracle_mod, pkg, mode):
    n = 400
    A, B = pkg.workloads.svd_conditioned(n, 2, cond=1e6, seed=3)
    f = ctx.factor(n, n, "fp32")
    assert f.getrf(A) == 0
    X, st = f.solve_refined(B, mode=mode)
    be = oracle_mod.backward_error(A, X, B)
    assert be <= 10 * n * EPS64, (be, st)
    f.close()


def test_transposed_refined(ctx, oracle_mod, pkg):
    n = 300
    A, B = pkg.workloads.shifted(n, 2, seed=5)
    f = ctx.factor(n, n, "fp32")
    f.getrf(A)
    X, st = f.solve_refined(B, trans="T")
    assert oracle_mod.backward_error(A.T, X, B) <= 10 * n * EPS64


def test_stall_falls_back_to_fp64(ctx, oracle_mod, pkg):
    # max_iter = 0 cannot converge: the FP64 LU must produce the answer
    n = 200
    A, B = pkg.workloads.plain(n, 2, seed=6)
    f = ctx.factor(n, n, "fp32")
    f.getrf(A)
    X, st = f.solve_refined(B, max_iter=0)
    assert st["fell_back"] == 1
    LU, ipiv, _ = oracle_mod.getrf(A)
    assert np.array_equal(X, oracle_mod.getrs(LU, ipiv, B))


def test_stall_without_fallback_errors(ctx, pkg):
    n = 100
    A, B = pkg.workloads.plain(n, 1, seed=7)
    f = ctx.factor(n, n, "fp32")
    f.getrf(A)
    with pytest.raises(pkg.GBLUError) as ei:
        f.solve_refined(B, max_iter=0, fallback=False)
    assert ei.value.status == 6  # GBLU_ESTALL


def test_default_getrs_is_refined(ctx, oracle_mod, pkg):
    n = 256
    A, B = pkg.workloads.plain(n, 3, seed=8)
    f = ctx.factor(n, n, "fp32")
    f.getrf(A)
    X = f.getrs(B)
    assert oracle_mod.backward_error(A, X, B) <= 10 * n * EPS64


def test_fp32_factors_bit_exact(ctx, oracle_mod, pkg):
    # the FP32 factorization follows the same per-element order in FP32
    n = 333
    A, _ = pkg.workloads.shifted(n, 1, seed=9)
    f = ctx.factor(n, n, "fp32")
    f.getrf(A)
    LU, ipiv, _ = oracle_mod.getrf(A.astype(np.float32))
    assert np.array_equal(f.ipiv(), ipiv)
    assert np.array_equal(f.factors(), LU.astype(np.float64))
