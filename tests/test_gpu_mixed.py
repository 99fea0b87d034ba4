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


@pytest.fixture(scope="module")
def kappa_1e6_n4096(pkg):
    # A = Q1 diag(s) Q2^T, s log-spaced 1..1e6 (the hard mixed configuration
    # at a quarter of its size), generated with FP64 QR on the GPU
    return pkg.workloads.svd_conditioned_gpu(4096, 4, cond=1e6, seed=21)


@pytest.fixture(scope="module")
def kappa_1e6_fp64_solution(ctx, kappa_1e6_n4096):
    A, B = kappa_1e6_n4096
    f = ctx.factor(4096, 4096, "fp64")
    assert f.getrf(A) == 0
    X = f.getrs(B)
    f.close()
    return X


@pytest.mark.parametrize("mode", ["ir", "gmres_ir"])
def test_kappa_1e6_n4096(ctx, oracle_mod, kappa_1e6_n4096, kappa_1e6_fp64_solution, mode):
    """FP32 LU + FP64 IR / GMRES-IR on a cond = 1e6 matrix of n = 4096 meets
    the 10 n eps64 backward-error bound; GMRES-IR needs no fallback; a column
    the fallback produced is the plain FP64 LU's answer bit for bit."""
    A, B = kappa_1e6_n4096
    n = A.shape[0]
    f = ctx.factor(n, n, "fp32")
    assert f.getrf(A) == 0
    X, st = f.solve_refined(B, mode=mode)
    be = oracle_mod.backward_error(A, X, B)
    assert be <= 10 * n * EPS64, (be, st)
    if mode == "gmres_ir":
        assert st["fell_back"] == 0 and st["converged"] == 1, st
    if st["fell_back"]:
        X64 = kappa_1e6_fp64_solution
        for j in range(B.shape[1]):
            ok = np.array_equal(X[:, j], X64[:, j])
            assert ok or oracle_mod.backward_error(A, X[:, j], B[:, j]) <= n * EPS64
    f.close()


def test_kappa_1e6_n4096_forced_fallback_bit_exact(ctx, kappa_1e6_n4096, kappa_1e6_fp64_solution):
    """With no refinement allowed every column falls back, and the answer is
    the plain FP64 LU's, bit for bit."""
    A, B = kappa_1e6_n4096
    n = A.shape[0]
    f = ctx.factor(n, n, "fp32")
    assert f.getrf(A) == 0
    X, st = f.solve_refined(B, max_iter=0)
    assert st["fell_back"] == 1
    assert np.array_equal(X, kappa_1e6_fp64_solution)
    f.close()


@pytest.mark.parametrize("prec", ["fp32", "bf16", "fp16"])
def test_pivot_growth_goes_to_fp64_at_once(ctx, oracle_mod, pkg, prec):
    """Wilkinson's matrix (growth 2^(n-1) under partial pivoting): the device
    computes the growth at getrf, the solve skips refinement and answers with
    the plain FP64 LU, bit for bit; without fallback it is GBLU_ESTALL."""
    n = 60
    A, B = pkg.workloads.growth_matrix(n, 2, seed=1)
    f = ctx.factor(n, n, prec)
    assert f.getrf(A) == 0
    assert f.growth() == 2.0 ** (n - 1)
    X, st = f.solve_refined(B)
    assert st["fell_back"] == 1 and st["fallback_reason"] == pkg._lib.GBLU_FALLBACK_GROWTH, st
    assert st["iterations"] == 0 and st["growth"] == 2.0 ** (n - 1)
    LU, ipiv, _ = oracle_mod.getrf(A)
    assert np.array_equal(X, oracle_mod.getrs(LU, ipiv, B))
    with pytest.raises(pkg.GBLUError) as ei:
        f.solve_refined(B, fallback=False)
    assert ei.value.status == 6  # GBLU_ESTALL
    f.close()


def test_growth_limit_option(ctx, oracle_mod, pkg):
    """A benign matrix has growth O(1) and refines; a growth_limit below its
    growth sends the same solve to the FP64 LU."""
    n = 500
    A, B = pkg.workloads.shifted(n, 2, seed=31)
    f = ctx.factor(n, n, "fp32")
    assert f.getrf(A) == 0
    g = f.growth()
    assert 0.5 <= g <= 2.0, g
    X, st = f.solve_refined(B)
    assert st["fell_back"] == 0 and st["fallback_reason"] == 0 and st["growth"] == g
    X2, st2 = f.solve_refined(B, growth_limit=0.25)
    assert st2["fell_back"] == 1 and st2["fallback_reason"] == pkg._lib.GBLU_FALLBACK_GROWTH
    LU, ipiv, _ = oracle_mod.getrf(A)
    assert np.array_equal(X2, oracle_mod.getrs(LU, ipiv, B))
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


def _round_bf16(x):
    x = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _fp16_scaled(B):
    B = np.asarray(B, dtype=np.float32)
    mx = np.abs(B).max(axis=0)
    e = np.where(mx > 0, np.frexp(mx)[1] - 1 - 14, 0)  # ilogb(mx) - 14
    s = np.ldexp(np.float32(1.0), -e).astype(np.float32)
    Bh = (B * s).astype(np.float16).astype(np.float64)
    return Bh / s.astype(np.float64)


@pytest.mark.parametrize("prec", ["bf16", "fp16", "fp32"])
@pytest.mark.parametrize("m,n,k", [(5, 7, 3), (128, 128, 64), (129, 130, 65), (300, 200, 100),
                                   (1000, 513, 777), (256, 384, 1024),
                                   # enough 128 x 256 tiles to cover the SMs: the wide-tile kernel,
                                   # also with ragged edges in every dimension
                                   (4096, 2560, 192), (4001, 2600, 100)])
def test_gemm_update_against_rounded_operands(ctx, prec, m, n, k):
    """The trailing-update contraction: C - A B with 16-bit operands and FP32
    accumulation (tcgen05), checked against float64 products of the rounded
    operands; FP32 mode is checked the same way with unrounded operands."""
    rng = np.random.default_rng(m * 7 + n * 3 + k)
    A = rng.uniform(-1, 1, size=(m, k)).astype(np.float32)      # |L21| <= 1
    B = (rng.standard_normal((k, n)) * 37.0).astype(np.float32)  # U12-like
    C = rng.standard_normal((m, n)).astype(np.float32)
    out = ctx.gemm_update(C, A, B, prec)
    if prec == "bf16":
        Ar, Br = _round_bf16(A), _round_bf16(B)
    elif prec == "fp16":
        Ar, Br = A.astype(np.float16).astype(np.float64), _fp16_scaled(B)
    else:
        Ar, Br = A.astype(np.float64), B.astype(np.float64)
    ref = C.astype(np.float64) - Ar @ Br
    scale = np.abs(Ar) @ np.abs(Br) + np.abs(C)
    err = np.abs(out.astype(np.float64) - ref) / scale
    assert err.max() < 4 * (k + 2) * 2.0 ** -24, err.max()


@pytest.mark.parametrize("prec", ["bf16", "fp16"])
@pytest.mark.parametrize("mode", ["ir", "gmres_ir"])
@pytest.mark.parametrize("n", [256, 1000, 2048])
def test_tensor_core_lu_reaches_fp64(ctx, oracle_mod, pkg, prec, mode, n):
    A, B = pkg.workloads.shifted(n, 2, seed=100 + n)
    f = ctx.factor(n, n, prec)
    assert f.getrf(A) == 0
    X, st = f.solve_refined(B, mode=mode)
    be = oracle_mod.backward_error(A, X, B)
    assert be <= 10 * n * EPS64, (be, st)
    assert st["fell_back"] == 0, st
    # the 16-bit-operand factors (TRSM base blocks through cached inverses)
    # factor A: P A = L U up to the 16-bit operand rounding
    _check_factorization(A, f.factors(), f.ipiv(), 0.05)
    f.close()


def _check_factorization(A, F, ipiv, tol):
    """ipiv is a valid 1-based interchange sequence and P A = L U within tol
    (relative to max |A|)."""
    n = A.shape[0]
    assert all(k + 1 <= int(p) <= n for k, p in enumerate(ipiv))
    PA = np.array(A, dtype=np.float64, copy=True)
    for k, p in enumerate(ipiv):
        if p - 1 != k:
            PA[[k, p - 1], :] = PA[[p - 1, k], :]
    L = np.tril(F, -1) + np.eye(n)
    U = np.triu(F)
    err = np.abs(PA - L @ U).max() / np.abs(A).max()
    assert err < tol, err
    return err


def _factor_error(ctx, monkeypatch, A, prec, panel, env="GBLU_PANEL"):
    monkeypatch.setenv(env, panel)  # read when the factor is created
    n = A.shape[0]
    f = ctx.factor(n, n, prec)
    monkeypatch.delenv(env)
    assert f.getrf(A) == 0
    F, ipiv = f.factors(), f.ipiv()
    f.close()
    return _check_factorization(A, F, ipiv, 1.0), np.abs(np.tril(F, -1)).max(), ipiv


def test_tournament_panel_fp32_factors(ctx, pkg, monkeypatch):
    """The tournament panel on FP32 factors (GBLU_PANEL=tournament), where
    the factorization error is at FP32 level: P A = L U as accurately as with
    partial pivoting, valid interchanges that do move rows, bounded
    multipliers -- the row moves and L21 = A21 U11^-1 are checked exactly
    enough to expose any misplaced row."""
    A, _ = pkg.workloads.plain(2500, 1, seed=72)
    e_t, lmax_t, ipiv_t = _factor_error(ctx, monkeypatch, A, "fp32", "tournament")
    e_p, lmax_p, ipiv_p = _factor_error(ctx, monkeypatch, A, "fp32", "partial")
    assert lmax_p <= 1.0 and lmax_t < 16.0
    assert (ipiv_t != np.arange(1, 2501)).sum() > 1000  # pivots move rows
    assert not np.array_equal(ipiv_t, ipiv_p)           # and differ from partial pivoting's
    assert e_t < 10 * e_p + 1e-6, (e_t, e_p)
    assert e_t < 1e-4, e_t


@pytest.mark.parametrize("prec", ["bf16", "fp16"])
def test_tournament_panel_factors_and_refines(ctx, oracle_mod, pkg, monkeypatch, prec):
    """Leaves taller than 512 rows of the 16-bit-operand factors pick their
    pivots by tournament (chunk factorizations, then one over the nominated
    rows): the factors are as accurate as partial pivoting's at the same
    operand precision, and refinement reaches the FP64 bound on shifted and
    on plain Gaussian matrices."""
    for A, B in (pkg.workloads.shifted(3000, 2, seed=71), pkg.workloads.plain(2500, 2, seed=72)):
        n = A.shape[0]
        e_t, lmax_t, _ = _factor_error(ctx, monkeypatch, A, prec, "tournament")
        e_p, _, _ = _factor_error(ctx, monkeypatch, A, prec, "partial")
        assert e_t < 3 * e_p + 1e-3, (e_t, e_p)
        assert lmax_t < 16.0
        monkeypatch.setenv("GBLU_PANEL", "tournament")
        f = ctx.factor(n, n, prec)
        monkeypatch.delenv("GBLU_PANEL")
        assert f.getrf(A) == 0
        X, st = f.solve_refined(B, mode="gmres_ir")
        assert oracle_mod.backward_error(A, X, B) <= 10 * n * EPS64, st
        f.close()


def test_tournament_panel_off_switch(ctx, oracle_mod, pkg, monkeypatch):
    """GBLU_PANEL=partial at factor creation keeps partial pivoting for the
    16-bit-operand factors: every multiplier is then at most 1."""
    monkeypatch.setenv("GBLU_PANEL", "partial")
    n = 1500
    A, B = pkg.workloads.plain(n, 1, seed=73)
    f = ctx.factor(n, n, "bf16")
    assert f.getrf(A) == 0
    F = f.factors()
    assert np.abs(np.tril(F, -1)).max() <= 1.0
    X, st = f.solve_refined(B, mode="gmres_ir")
    assert oracle_mod.backward_error(A, X, B) <= 10 * n * EPS64, st
    f.close()


def test_tensor_core_lu_ill_conditioned_gmres(ctx, oracle_mod, pkg):
    n = 600
    A, B = pkg.workloads.svd_conditioned(n, 2, cond=1e4, seed=11)
    f = ctx.factor(n, n, "fp16")
    assert f.getrf(A) == 0
    X, st = f.solve_refined(B, mode="gmres_ir")
    assert oracle_mod.backward_error(A, X, B) <= 10 * n * EPS64, st


@pytest.mark.parametrize("n", [1000, 2048])
def test_trsm_inverse_blocks(ctx, oracle_mod, pkg, monkeypatch, n):
    """The 16-bit-operand factors solve TRSM base blocks of 65..128 rows
    through cached inverses of L's diagonal blocks: factors as accurate as
    with the substitution chain (GBLU_TRSM=exact), for power-of-two and
    uneven recursion splits, and refinement reaches the FP64 bound."""
    A, B = pkg.workloads.plain(n, 2, seed=90 + n)
    e_inv, _, ipiv_inv = _factor_error(ctx, monkeypatch, A, "bf16", "default", env="GBLU_TRSM")
    e_chain, _, ipiv_chain = _factor_error(ctx, monkeypatch, A, "bf16", "exact", env="GBLU_TRSM")
    assert e_inv < 2 * e_chain + 1e-3, (e_inv, e_chain)
    f = ctx.factor(n, n, "bf16")
    assert f.getrf(A) == 0
    X, st = f.solve_refined(B, mode="gmres_ir")
    assert oracle_mod.backward_error(A, X, B) <= 10 * n * EPS64, st
    f.close()


def _rbt_diagonals(n):
    """The butterflies' random diagonals as the library draws them: a
    splitmix64 stream from a fixed seed, exp(u / 10) with u uniform in
    (-1/2, 1/2), rounded to FP32; left then right, each R1 S1 R2 S2 of n4/2
    (n4 = n - n mod 4, the order the butterflies cover)."""
    n4 = n - n % 4
    mask = (1 << 64) - 1
    x = 0x5eedb077e4f1
    out = np.empty(4 * n4, dtype=np.float32)
    for i in range(4 * n4):
        x = (x + 0x9e3779b97f4a7c15) & mask
        z = x
        z = ((z ^ (z >> 30)) * 0xbf58476d1ce4e5b9) & mask
        z = ((z ^ (z >> 27)) * 0x94d049bb133111eb) & mask
        z ^= z >> 31
        u = (z >> 11) * (1.0 / 9007199254740992.0) - 0.5
        out[i] = np.float32(np.exp(u / 10.0))
    return out


def _rbt_matrices(n):
    """U = diag(W_L / 2, I) and V = diag(W_R / 2, I): the factors are those of
    U^T A V."""
    d = _rbt_diagonals(n).astype(np.float64)
    n4 = n - n % 4
    h1, h2 = n4 // 2, n4 // 4

    def butterfly(R, S):
        m = 2 * len(R)
        B = np.zeros((m, m))
        B[:m // 2, :m // 2] = np.diag(R)
        B[:m // 2, m // 2:] = np.diag(S)
        B[m // 2:, :m // 2] = np.diag(R)
        B[m // 2:, m // 2:] = -np.diag(S)
        return B

    Ts = []
    for side in (0, 1):
        b = d[side * 2 * n4:(side + 1) * 2 * n4]
        R1, S1, R2, S2 = b[:h1], b[h1:n4], b[n4:n4 + h1], b[n4 + h1:]
        B2 = np.zeros((n4, n4))
        B2[:h1, :h1] = butterfly(R2[:h2], S2[:h2])
        B2[h1:, h1:] = butterfly(R2[h2:], S2[h2:])
        T = np.eye(n)
        T[:n4, :n4] = butterfly(R1, S1) @ B2 / 2
        Ts.append(T)
    return Ts


@pytest.mark.parametrize("prec", ["fp32", "bf16", "fp16"])
@pytest.mark.parametrize("n", [256, 1000, 1001, 1002, 1003, 7])
def test_rbt_factors_the_transformed_matrix(ctx, oracle_mod, pkg, prec, n):
    """GBLU_PIVOT_RBT: the low-precision LU is that of U^T A V (the
    butterflies rebuilt here from the library's seeded diagonals; for n not a
    multiple of 4 the last n mod 4 rows and columns are left out of them),
    without interchanges, and refinement reaches the FP64 bound without
    fallback."""
    # A = G + 4 sqrt(n) I: the transform keeps the growth near 1 (GENP on a
    # plain Gaussian matrix meets small pivots whatever the randomisation)
    A, B = pkg.workloads.shifted(n, 3, seed=300 + n)
    f = ctx.factor(n, n, prec)
    f.set_pivoting("rbt")
    assert f.getrf(A) == 0
    U_, V_ = _rbt_matrices(n)
    Ar = U_.T @ A @ V_
    F = f.factors()
    L = np.tril(F, -1) + np.eye(n)
    U = np.triu(F)
    assert np.array_equal(f.ipiv(), np.arange(1, n + 1))
    err = np.abs(Ar - L @ U).max() / np.abs(Ar).max()
    assert err < {"fp32": 1e-4, "bf16": 0.1, "fp16": 0.02}[prec], err
    X, st = f.solve_refined(B, mode="ir")
    assert oracle_mod.backward_error(A, X, B) <= 10 * n * EPS64, st
    assert st["fell_back"] == 0, st
    Xt, st = f.solve_refined(B, trans="T", mode="gmres_ir")
    assert oracle_mod.backward_error(A.T, Xt, B) <= 10 * n * EPS64, st
    assert st["fell_back"] == 0, st
    f.close()


def test_rbt_plain_gaussian_gmres(ctx, oracle_mod, pkg):
    """A plain Gaussian matrix: no pivoting meets small pivots (growth in the
    thousands, measured on the host for this construction); FP32 GMRES-IR
    still reaches the FP64 bound, and the growth is reported."""
    n = 1000
    A, B = pkg.workloads.plain(n, 2, seed=1300)
    f = ctx.factor(n, n, "fp32")
    f.set_pivoting("rbt")
    assert f.getrf(A) == 0
    X, st = f.solve_refined(B, mode="gmres_ir")
    assert oracle_mod.backward_error(A, X, B) <= 10 * n * EPS64, st
    assert st["growth"] > 10, st
    f.close()


def test_rbt_kappa_1e6_n4096(ctx, oracle_mod, kappa_1e6_n4096):
    """The κ = 1e6 matrix, FP32 LU without pivoting after the transform,
    GMRES-IR: the no-pivot factors (growth in the hundreds here) are too weak
    a preconditioner for this conditioning, refinement stalls and the FP64
    fallback delivers the FP64 bound."""
    A, B = kappa_1e6_n4096
    n = A.shape[0]
    f = ctx.factor(n, n, "fp32")
    f.set_pivoting("rbt")
    assert f.getrf(A) == 0
    X, st = f.solve_refined(B, mode="gmres_ir")
    assert oracle_mod.backward_error(A, X, B) <= 10 * n * EPS64, st
    assert st["growth"] > 10, st
    f.close()


def test_rbt_mode_switches_and_graph_replay(ctx, oracle_mod, pkg):
    """Switching the pivoting invalidates the factors (solves report
    GBLU_ENOTFACTORED until the next getrf); repeated RBT getrfs (replayed
    from the captured launch sequence from the third on) stay correct, and so
    does partial pivoting after switching back."""
    n = 768
    f = ctx.factor(n, n, "bf16")
    for mode in ("rbt", "partial", "rbt"):
        f.set_pivoting(mode)
        with pytest.raises(pkg.GBLUError):
            f.solve_refined(np.ones((n, 1)))
        for rep in range(4):
            A, B = pkg.workloads.shifted(n, 2, seed=500 + rep)
            assert f.getrf(A) == 0
            X, st = f.solve_refined(B)
            assert oracle_mod.backward_error(A, X, B) <= 10 * n * EPS64, (mode, rep, st)
            assert st["fell_back"] == 0
    f.close()


def test_rbt_needs_a_square_mixed_factor(ctx, pkg):
    """RBT takes mixed factors (square by construction) of order 4 or more,
    not FP64 ones."""
    for m, n, prec in ((3, 3, "bf16"), (2, 2, "fp32"), (64, 64, "fp64")):
        f = ctx.factor(m, n, prec)
        with pytest.raises(pkg.GBLUError):
            f.set_pivoting("rbt")
        if prec != "fp64":
            f.set_pivoting("partial")
        f.close()


@pytest.mark.parametrize("pivot", ["partial", "rbt"])
def test_full_size_mixed_n16384(ctx, oracle_mod, pkg, pivot):
    """The mixed configuration at its full size (n = 16384, A = G + 4 sqrt(n) I,
    4 RHS): BF16 tcgen05 LU + FP64 IR within 10 n eps64 without fallback, for
    partial pivoting and for no pivoting after the butterfly transform."""
    n = 16384
    A, B = pkg.workloads.shifted(n, 4, seed=1)
    f = ctx.factor(n, n, "bf16")
    f.set_pivoting(pivot)
    assert f.getrf(A) == 0
    X, st = f.solve_refined(B)
    be = oracle_mod.backward_error(A, X, B)
    assert be <= 10 * n * EPS64, (be, st)
    assert st["fell_back"] == 0, st
    f.close()
