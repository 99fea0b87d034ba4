"""The oracle pinned against the reference's own test vectors and metrics and
against LAPACK getrf/getrs (the routines LUFactorization calls)."""
import numpy as np
import pytest

from conftest import EPS64


def test_known_answer(oracle_mod, golden):
    # test/Core/resolve.jl:78-106
    LU, ipiv, info = oracle_mod.getrf(golden["known_A"])
    assert info == 0
    x = oracle_mod.getrs(LU, ipiv, golden["known_b"])
    np.testing.assert_allclose(x, golden["known_x"], rtol=1e-12, atol=1e-12)


def test_matches_lapack_golden(oracle_mod, golden):
    for key in golden["cases"]:
        A = golden[key + "_A"]
        LU, ipiv, info = oracle_mod.getrf(A)
        assert info == int(golden[key + "_info"])
        assert np.array_equal(ipiv, golden[key + "_ipiv"]), key
        scale = max(1.0, np.abs(golden[key + "_LU"]).max())
        assert np.abs(LU - golden[key + "_LU"]).max() <= 1e-11 * scale, key
        if key + "_b" in golden:
            x = oracle_mod.getrs(LU, ipiv, golden[key + "_b"])
            np.testing.assert_allclose(x, golden[key + "_x"], rtol=1e-9, atol=1e-12)
            xt = oracle_mod.getrs(LU, ipiv, golden[key + "_b"], trans="T")
            np.testing.assert_allclose(xt, golden[key + "_xt"], rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_scaled_residual_square(oracle_mod, dtype):
    # test/Core/blocked_lufact.jl:44-54: scaled residual < 20
    rng = np.random.default_rng(1234)
    for n in (1, 2, 3, 5, 7, 8, 9, 13, 16, 17, 31, 32, 33, 40, 41, 63, 64, 65,
              100, 127, 128, 129, 200, 250, 256, 257, 300):
        A = rng.standard_normal((n, n)).astype(dtype)
        LU, ipiv, info = oracle_mod.getrf(A)
        assert info == 0
        assert oracle_mod.scaled_residual(A, LU, ipiv) < 20, n


def test_rectangular(oracle_mod):
    # test/Core/blocked_lufact.jl:119-130
    rng = np.random.default_rng(5)
    for m, n in ((100, 3), (3, 100), (128, 40), (40, 128), (257, 130), (130, 257), (65, 64), (64, 65)):
        A = rng.standard_normal((m, n))
        LU, ipiv, info = oracle_mod.getrf(A)
        assert oracle_mod.scaled_residual(A, LU, ipiv) < 20


def test_panel_width_invariance(oracle_mod):
    # each element sees fma(-l, u, a) for k ascending whatever the blocking,
    # so every panel width gives the same bits (test/Core/blocked_lufact.jl:56-70)
    rng = np.random.default_rng(9)
    for n in (11, 41, 67, 97, 130):
        A = rng.standard_normal((n, n))
        ref = oracle_mod.getrf(A)
        for nb in (1, 4, 5, 8, 13, 16, 32):
            got = oracle_mod.getrf_nb(A, nb)
            assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1]), (n, nb)


def test_singular_info(oracle_mod, golden):
    # test/Core/lu_refactorization.jl:83-110: zero first column -> info = 1
    LU, ipiv, info = oracle_mod.getrf(golden["sing_A"])
    assert info == int(golden["sing_info"]) == 1
    LU, ipiv, info = oracle_mod.getrf(golden["sing_Agood"])
    assert info == 0


def test_backward_error_metric(oracle_mod):
    rng = np.random.default_rng(3)
    n = 200
    A = rng.standard_normal((n, n))
    b = rng.standard_normal(n)
    LU, ipiv, _ = oracle_mod.getrf(A)
    x = oracle_mod.getrs(LU, ipiv, b)
    assert oracle_mod.backward_error(A, x, b) <= 10 * n * EPS64
    x_lapack, _ = oracle_mod.lapack_solve(A, b)
    assert oracle_mod.forward_error(x, x_lapack) < 1e-10


def test_batched_oracle(oracle_mod, pkg):
    sizes, A, b, _ = pkg.workloads.batch(12, seed=4)
    Aout, X, info = oracle_mod.gesv_batched(sizes, A, b)
    a_off, b_off = pkg.workloads.offsets(sizes)
    for i, n in enumerate(sizes):
        n = int(n)
        Ai = A[a_off[i]:a_off[i] + n * n].reshape(n, n, order="F")
        xi = X[b_off[i]:b_off[i] + n]
        bi = b[b_off[i]:b_off[i] + n]
        assert info[i] == 0
        assert oracle_mod.backward_error(Ai, xi, bi) <= 10 * n * EPS64


def test_luflop_matches_reference_function(oracle_mod):
    # benchmarks/lu.jl:8-20 evaluated literally for small sizes
    def ref(m, n):
        total = 0
        for k in range(1, min(m, n) + 1):
            scale = sum(range(k + 1, m + 1))
            upd = sum(2 for j in range(k + 1, n + 1) for i in range(k + 1, m + 1))
            total += 1 + scale + upd
        return total
    for m, n in ((1, 1), (5, 5), (7, 4), (4, 7), (30, 30)):
        assert oracle_mod.luflop(m, n) == ref(m, n)
