"""getrf / getrs on the GPU against the oracle (bit-exact) and LAPACK.

The GPU factorization keeps the reference's per-element operation order, so
ipiv and the packed factors must equal the C restatement of
src/blocked_lufact.jl bit for bit, and the solve must equal the restated
src/factorization.jl:433-457 back-solve bit for bit."""
import numpy as np
import pytest

from conftest import EPS64

pytestmark = pytest.mark.gpu

SQUARE = [1, 2, 3, 5, 7, 8, 9, 13, 16, 17, 31, 32, 33, 40, 41, 63, 64, 65, 100, 127, 128, 129,
          200, 250, 256, 257, 300, 500, 512, 1000]


@pytest.mark.parametrize("n", SQUARE)
def test_getrf_bit_exact(ctx, oracle_mod, n):
    rng = np.random.default_rng(1000 + n)
    A = rng.standard_normal((n, n))
    f = ctx.factor(n, n)
    info = f.getrf(A)
    LU, ipiv, info_ref = oracle_mod.getrf(A)
    assert info == info_ref == 0
    assert np.array_equal(f.ipiv(), ipiv)
    assert np.array_equal(f.factors(), LU)
    f.close()


@pytest.mark.parametrize("m,n", [(100, 3), (3, 100), (128, 40), (40, 128), (257, 130), (130, 257),
                                 (65, 64), (64, 65), (513, 100), (100, 513), (2000, 70)])
def test_getrf_rectangular_bit_exact(ctx, oracle_mod, m, n):
    rng = np.random.default_rng(m * 1000 + n)
    A = rng.standard_normal((m, n))
    f = ctx.factor(m, n)
    f.getrf(A)
    LU, ipiv, info_ref = oracle_mod.getrf(A)
    assert np.array_equal(f.ipiv(), ipiv)
    assert np.array_equal(f.factors(), LU)
    assert oracle_mod.scaled_residual(A, f.factors(), f.ipiv()) < 20
    f.close()


def test_getrf_matches_lapack_golden(ctx, golden):
    for key in golden["cases"]:
        A = golden[key + "_A"]
        m, n = A.shape
        f = ctx.factor(m, n)
        info = f.getrf(A)
        assert info == int(golden[key + "_info"])
        assert np.array_equal(f.ipiv(), golden[key + "_ipiv"]), key
        scale = max(1.0, np.abs(golden[key + "_LU"]).max())
        assert np.abs(f.factors() - golden[key + "_LU"]).max() <= 1e-11 * scale
        if key + "_b" in golden:
            np.testing.assert_allclose(f.getrs(golden[key + "_b"]), golden[key + "_x"], rtol=1e-9,
                                       atol=1e-12)
            np.testing.assert_allclose(f.getrs(golden[key + "_b"], trans="T"), golden[key + "_xt"],
                                       rtol=1e-9, atol=1e-12)
        f.close()


@pytest.mark.parametrize("n", [1, 5, 63, 64, 65, 127, 200, 513, 1000])
@pytest.mark.parametrize("nrhs", [1, 3, 8, 11])
def test_getrs_bit_exact(ctx, oracle_mod, n, nrhs):
    rng = np.random.default_rng(n * 31 + nrhs)
    A = rng.standard_normal((n, n))
    B = rng.standard_normal((n, nrhs))
    f = ctx.factor(n, n)
    f.getrf(A)
    LU, ipiv, _ = oracle_mod.getrf(A)
    X = f.getrs(B)
    assert np.array_equal(X, oracle_mod.getrs(LU, ipiv, B))
    XT = f.getrs(B, trans="T")
    assert np.array_equal(XT, oracle_mod.getrs(LU, ipiv, B, trans="T"))
    assert oracle_mod.backward_error(A, X, B) <= 10 * n * EPS64
    assert oracle_mod.backward_error(A.T, XT, B) <= 10 * n * EPS64
    f.close()


def test_known_answer(ctx, golden):
    f = ctx.factor(2, 2)
    f.getrf(golden["known_A"])
    np.testing.assert_allclose(f.getrs(golden["known_b"]), golden["known_x"], rtol=1e-12)
    f.close()


def test_singular_zero_column(ctx, oracle_mod, golden):
    f = ctx.factor(8, 8)
    info = f.getrf(golden["sing_A"])
    LU, ipiv, info_ref = oracle_mod.getrf(golden["sing_A"])
    assert info == info_ref == 1
    assert np.array_equal(f.ipiv(), ipiv)
    assert np.array_equal(f.factors(), LU)
    # solving with a singular factorization is refused, not silently wrong
    with pytest.raises(Exception):
        f.getrs(np.ones(8))
    # the same object recovers on the next nonsingular matrix
    assert f.getrf(golden["sing_Agood"]) == 0
    x = f.getrs(np.ones(8))
    assert oracle_mod.backward_error(golden["sing_Agood"], x, np.ones(8)) <= 80 * EPS64
    f.close()


def test_zero_pivot_later_column(ctx, oracle_mod):
    # rank-deficient: column 5 a combination of columns 0..4 -> exact zero pivot possible
    rng = np.random.default_rng(11)
    n = 70
    A = rng.integers(-3, 4, size=(n, n)).astype(np.float64)
    A[:, 40] = 0.0
    f = ctx.factor(n, n)
    info = f.getrf(A)
    LU, ipiv, info_ref = oracle_mod.getrf(A)
    assert info == info_ref and info > 0
    assert np.array_equal(f.ipiv(), ipiv)
    assert np.array_equal(f.factors(), LU)
    f.close()


def test_ties_and_small_integers(ctx, oracle_mod):
    # many exactly equal |a| candidates: the first-index rule must match
    rng = np.random.default_rng(12)
    for n in (17, 96, 300):
        A = rng.choice([-2.0, -1.0, 1.0, 2.0], size=(n, n))
        f = ctx.factor(n, n)
        info = f.getrf(A)
        LU, ipiv, info_ref = oracle_mod.getrf(A)
        assert info == info_ref
        assert np.array_equal(f.ipiv(), ipiv)
        assert np.array_equal(f.factors(), LU)
        f.close()


def test_nan_input_propagates(ctx, oracle_mod):
    rng = np.random.default_rng(13)
    n = 50
    A = rng.standard_normal((n, n))
    A[7, 3] = np.nan
    f = ctx.factor(n, n)
    info = f.getrf(A)
    LU, ipiv, info_ref = oracle_mod.getrf(A)
    assert info == info_ref
    assert np.array_equal(f.ipiv(), ipiv)
    np.testing.assert_array_equal(np.isnan(f.factors()), np.isnan(LU))
    f.close()


def test_empty(ctx):
    f = ctx.factor(0, 0)
    assert f.getrf(np.zeros((0, 0))) == 0
    f.close()


def test_factor_reuse_no_reallocation(ctx, oracle_mod):
    # refactor cycles A2, A1, A2 on one factor object (test/Core/lu_refactorization.jl:28-66)
    rng = np.random.default_rng(14)
    n = 51
    A1 = rng.random((n, n)) + n * np.eye(n)
    A2 = rng.random((n, n)) + n * np.eye(n)
    b = rng.random(n)
    f = ctx.factor(n, n)
    f.getrf(A1)
    f.getrs(b)
    used = ctx.memory()[0]
    for Ak in (A2, A1, A2):
        assert f.getrf(Ak) == 0
        x = f.getrs(b)
        LU, ipiv, _ = oracle_mod.getrf(Ak)
        assert np.array_equal(x, oracle_mod.getrs(LU, ipiv, b))
        assert ctx.memory()[0] == used  # refactor + solve allocate nothing
    f.close()


@pytest.mark.parametrize("n", [2048])
def test_getrf_bit_exact_medium(ctx, oracle_mod, n):
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n))
    f = ctx.factor(n, n)
    f.getrf(A)
    LU, ipiv, _ = oracle_mod.getrf(A)
    assert np.array_equal(f.ipiv(), ipiv)
    assert np.array_equal(f.factors(), LU)
    b = rng.standard_normal(n)
    assert np.array_equal(f.getrs(b), oracle_mod.getrs(LU, ipiv, b))
    f.close()


def test_full_size_config_backward_error(ctx, oracle_mod, pkg):
    # n = 8192, 16 RHS through one factorization: the size-independent bound
    n = 8192
    A, B = pkg.workloads.plain(n, 16, seed=0)
    f = ctx.factor(n, n)
    assert f.getrf(A) == 0
    X = f.getrs(B)
    be = oracle_mod.backward_error(A, X, B)
    assert be <= 10 * n * EPS64, be
    # forward error against the LAPACK solve of the same system, reported
    Xl, _ = oracle_mod.lapack_solve(A, B)
    fe = oracle_mod.forward_error(X, Xl)
    print(f"n={n}: backward error {be:.3e}, forward error vs LAPACK {fe:.3e}")
    assert fe < 1e-6
    f.close()


def test_lapack_shaped_entries(pkg, oracle_mod):
    rng = np.random.default_rng(15)
    for (m, n) in ((40, 40), (130, 70), (70, 130)):
        A = rng.standard_normal((m, n))
        LU, ipiv, info = pkg.dgetrf(A)
        LUo, ipivo, infoo = oracle_mod.getrf(A)
        assert info == infoo
        assert np.array_equal(ipiv, ipivo) and np.array_equal(LU, LUo)
    A = rng.standard_normal((90, 90))
    LU, ipiv, info = oracle_mod.getrf(A)
    B = rng.standard_normal((90, 3))
    assert np.array_equal(pkg.dgetrs(LU, ipiv, B), oracle_mod.getrs(LU, ipiv, B))
    assert np.array_equal(pkg.dgetrs(LU, ipiv, B, "T"), oracle_mod.getrs(LU, ipiv, B, "T"))


def test_lapack_shaped_single(pkg, oracle_mod):
    import ctypes
    lib = pkg.load_library()
    rng = np.random.default_rng(16)
    n = 77
    A = np.asfortranarray(rng.standard_normal((n, n)).astype(np.float32))
    LU = A.copy(order="F")
    ipiv = np.zeros(n, dtype=np.int64)
    m_, n_, lda, info = (ctypes.c_int64(n), ctypes.c_int64(n), ctypes.c_int64(n), ctypes.c_int64())
    lib.gblu_sgetrf_(ctypes.byref(m_), ctypes.byref(n_), LU.ctypes.data, ctypes.byref(lda),
                     ipiv.ctypes.data, ctypes.byref(info))
    LUo, ipivo, infoo = oracle_mod.getrf(A)
    assert info.value == infoo == 0
    assert np.array_equal(ipiv, ipivo) and np.array_equal(LU, LUo)
    b = np.asfortranarray(rng.standard_normal((n, 2)).astype(np.float32))
    x = b.copy(order="F")
    nrhs, ldb = ctypes.c_int64(2), ctypes.c_int64(n)
    lib.gblu_sgetrs_(b"N", ctypes.byref(n_), ctypes.byref(nrhs), LU.ctypes.data, ctypes.byref(lda),
                     ipiv.ctypes.data, x.ctypes.data, ctypes.byref(ldb), ctypes.byref(info), 1)
    assert info.value == 0
    assert np.array_equal(x, oracle_mod.getrs(LUo, ipivo, b))


def test_markstein_division_matches_ieee():
    """The back-solve divides by U[j,j] with Markstein's FMA-based division
    from a precomputed reciprocal; it must give the IEEE quotient bit for bit
    (2^26 random operand pairs per type, edge significands included)."""
    import ctypes
    import os
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    lib = ctypes.CDLL(os.path.join(root, "linearsolve.jl_gb300", "libgblu_tools.so"))
    lib.gblu_tool_divcheck.argtypes = [ctypes.c_int64, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64),
                                       ctypes.POINTER(ctypes.c_uint64)]
    lib.gblu_tool_divcheck.restype = ctypes.c_int32
    m64, m32 = ctypes.c_uint64(), ctypes.c_uint64()
    assert lib.gblu_tool_divcheck(1 << 26, 12345, ctypes.byref(m64), ctypes.byref(m32)) == 0
    assert m64.value == 0 and m32.value == 0, (m64.value, m32.value)


def test_f64_to_f32_conversion_matches_hardware():
    """The mixed factors convert A with an integer-pipe FP64 -> FP32 narrowing
    (round to nearest even); it must give the hardware conversion's result
    bit for bit (2^26 doubles: every exponent, the FP32 boundaries, rounding
    ties; NaNs by NaN-ness)."""
    import ctypes
    import os
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    lib = ctypes.CDLL(os.path.join(root, "linearsolve.jl_gb300", "libgblu_tools.so"))
    lib.gblu_tool_cvtcheck.argtypes = [ctypes.c_int64, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]
    lib.gblu_tool_cvtcheck.restype = ctypes.c_int32
    bad = ctypes.c_uint64()
    assert lib.gblu_tool_cvtcheck(1 << 26, 777, ctypes.byref(bad)) == 0
    assert bad.value == 0, bad.value


@pytest.mark.parametrize("kind", ["grid", "cluster", "reg"])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_every_panel_kernel_bit_exact(ctx, oracle_mod, monkeypatch, kind, prec):
    # the three getf2 kernels (cooperative grid, shared-memory cluster,
    # register cluster) give identical factors; GBLU_PANEL forces one of them
    monkeypatch.setenv("GBLU_PANEL", kind)
    rng = np.random.default_rng(77)
    shapes = ((700, 700), (1100, 300), (300, 520)) if prec == "fp64" else ((700, 700), (1300, 1300))
    for m, n in shapes:
        A = rng.standard_normal((m, n))
        dt = np.float32 if prec == "fp32" else np.float64
        f = ctx.factor(m, n, prec)
        f.getrf(A.astype(dt).astype(np.float64))
        LU, ipiv, _ = oracle_mod.getrf(A.astype(dt))
        assert np.array_equal(f.ipiv(), ipiv), (kind, prec, m, n)
        assert np.array_equal(f.factors(), LU.astype(np.float64)), (kind, prec, m, n)
        f.close()


@pytest.mark.parametrize("tile", ["128", "64", "32", "16"])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_every_gemm_tile_bit_exact(ctx, oracle_mod, monkeypatch, tile, prec):
    # the SIMT trailing update picks a 128 (FP32 register-blocked kernel), 64,
    # 32 or 16 square tile by shape; GBLU_GEMM_TILE forces one for every
    # update (same per-element order)
    monkeypatch.setenv("GBLU_GEMM_TILE", tile)
    rng = np.random.default_rng(79)
    dt = np.float32 if prec == "fp32" else np.float64
    shapes = ((1000, 1000), (1200, 700), (500, 900)) if prec == "fp64" else ((1000, 1000), (1300, 1300))
    for m, n in shapes:
        A = rng.standard_normal((m, n)).astype(dt).astype(np.float64)
        f = ctx.factor(m, n, prec)
        f.getrf(A)
        LU, ipiv, _ = oracle_mod.getrf(A.astype(dt))
        assert np.array_equal(f.ipiv(), ipiv), (tile, prec, m, n)
        assert np.array_equal(f.factors(), LU.astype(np.float64)), (tile, prec, m, n)
        f.close()


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_graph_replayed_getrf_matches_direct(ctx, oracle_mod, prec):
    # from its third factorization a factor replays its launch sequence from a
    # captured CUDA graph; new matrices must give the same bit-exact results
    n = 900
    rng = np.random.default_rng(88)
    dt = np.float32 if prec == "fp32" else np.float64
    f = ctx.factor(n, n, prec)
    for run in range(5):
        A = rng.standard_normal((n, n)).astype(dt).astype(np.float64)
        assert f.getrf(A) == 0
        LU, ipiv, _ = oracle_mod.getrf(A.astype(dt))
        assert np.array_equal(f.ipiv(), ipiv), run
        assert np.array_equal(f.factors(), LU.astype(np.float64)), run
    f.close()


# ---- fast getrs: inverted diagonal blocks (backward-error accurate) ----

@pytest.mark.parametrize("n", [1, 63, 64, 65, 200, 1000, 2049])
@pytest.mark.parametrize("nrhs", [1, 3, 11])
@pytest.mark.parametrize("trans", ["N", "T"])
def test_fast_getrs_backward_error(ctx, oracle_mod, n, nrhs, trans):
    """GBLU_SOLVE_FAST on FP64 factors: backward error within 10 n eps64 of
    op(A) and a solution close to the exact mode's, for ragged last blocks,
    several right-hand sides (more than one 8-column pass) and both
    orientations."""
    rng = np.random.default_rng(100 * n + nrhs)
    A = np.asfortranarray(rng.standard_normal((n, n)))
    B = np.asfortranarray(rng.standard_normal((n, nrhs)))
    f = ctx.factor(n, n, "fp64")
    assert f.getrf(A) == 0
    Xe = f.getrs(B, trans=trans)
    f.set_solve("fast")
    X = f.getrs(B, trans=trans)
    M = A if trans == "N" else A.T
    assert oracle_mod.backward_error(M, X, B) <= 10 * max(n, 1) * EPS64
    assert oracle_mod.forward_error(X, Xe) < 1e-8
    f.close()


def test_fast_getrs_follows_refactorization(ctx, oracle_mod):
    """The inverses are recomputed after each getrf: a new matrix in the same
    factor solves correctly, and exact mode can be switched back on."""
    n = 700
    f = ctx.factor(n, n, "fp64")
    f.set_solve("fast")
    for seed in (1, 2, 3):
        A = np.asfortranarray(np.random.default_rng(seed).standard_normal((n, n)))
        B = np.random.default_rng(seed + 10).standard_normal((n, 2))
        assert f.getrf(A) == 0
        assert oracle_mod.backward_error(A, f.getrs(B), B) <= 10 * n * EPS64
    f.set_solve("exact")
    LU, ipiv, _ = oracle_mod.getrf(A)
    assert np.array_equal(f.getrs(B), oracle_mod.getrs(LU, ipiv, B))
    f.close()


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
def test_fast_inner_solve_of_mixed_factors(ctx, oracle_mod, pkg, prec):
    n = 1500
    A, B = pkg.workloads.shifted(n, 4, seed=41)
    f = ctx.factor(n, n, prec)
    f.set_solve("fast")
    assert f.getrf(A) == 0
    for mode in ("ir", "gmres_ir"):
        X, st = f.solve_refined(B, mode=mode)
        assert oracle_mod.backward_error(A, X, B) <= 10 * n * EPS64, st
        assert st["fell_back"] == 0
    f.close()


def test_fast_getrs_through_the_interface(pkg, oracle_mod):
    rng = np.random.default_rng(43)
    n = 900
    A = rng.standard_normal((n, n))
    b = rng.standard_normal(n)
    cache = pkg.init(pkg.LinearProblem(A, b), pkg.GB300LUFactorization(solve="fast"))
    sol = pkg.solve_bang(cache)
    assert sol.retcode == pkg.ReturnCode.Success
    assert oracle_mod.backward_error(A, sol.u, b) <= 10 * n * EPS64
    cache.b = rng.standard_normal(n)
    sol = pkg.solve_bang(cache)
    assert oracle_mod.backward_error(A, sol.u, cache.b) <= 10 * n * EPS64


@pytest.mark.parametrize("pad", [0, 37])
def test_host_upload_staging_identical(pkg, pad):
    """Host matrices of 4 MB and more in pageable memory are copied through
    pinned staging chunks (here four 16 MB chunks, and a leading dimension
    above n); pinned host memory and device memory go straight to the copy
    engine.  All give identical factors, and a second staged upload in the
    same context (the chunks reused) too."""
    import ctypes
    import torch
    from importlib import import_module
    _lib = import_module(pkg.__name__ + "._lib")
    ctx = pkg.Context(0)
    n = 2600  # 54 MB: staged whatever else is in progress
    rng = np.random.default_rng(2600 + pad)
    Ap = np.asfortranarray(rng.standard_normal((n + pad, n)))  # pageable, lda = n + pad
    pinned = torch.empty((n, n + pad), dtype=torch.float64, pin_memory=True)
    pinned.numpy()[:] = Ap.T  # the same column-major matrix in pinned memory
    results = []
    for ptr in (Ap.ctypes.data, Ap.ctypes.data, pinned.data_ptr()):
        f = ctx.factor(n, n)
        info = ctypes.c_int64()
        st = ctx.lib.gblu_getrf(ctx.handle, f.handle, ptr, n + pad, _lib.GBLU_HOST, ctypes.byref(info))
        assert st == 0 and info.value == 0
        results.append((f.factors(), f.ipiv()))
        f.close()
    f = ctx.factor(n, n)
    dA = pkg.DeviceMatrix.from_host(np.asfortranarray(Ap[:n]))
    assert f.getrf(dA) == 0
    results.append((f.factors(), f.ipiv()))
    dA.free()
    f.close()
    ctx.close()
    for LU, ipiv in results[1:]:
        assert np.array_equal(LU, results[0][0]) and np.array_equal(ipiv, results[0][1])
