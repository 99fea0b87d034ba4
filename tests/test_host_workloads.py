"""The seeded synthetic inputs the tests and the bench share, checked on the
CPU: reproducible from their seed, column-major FP64, and with the property
each one is built for (the condition number of svd_conditioned, the 2^(n-1)
pivot growth of growth_matrix under partial pivoting, the batch's size
range and offsets)."""
import numpy as np
from scipy.linalg import lapack


def test_seeded_and_column_major(pkg):
    w = pkg.workloads
    for make in (w.plain, w.shifted):
        A1, B1 = make(50, 3, seed=7)
        A2, B2 = make(50, 3, seed=7)
        A3, _ = make(50, 3, seed=8)
        assert np.array_equal(A1, A2) and np.array_equal(B1, B2) and not np.array_equal(A1, A3)
        assert A1.dtype == np.float64 and A1.flags.f_contiguous and B1.shape == (50, 3)


def test_svd_conditioned_has_its_condition(pkg):
    A, B = pkg.workloads.svd_conditioned(200, 2, cond=1e6, seed=1)
    s = np.linalg.svd(A, compute_uv=False)
    assert abs(s[0] / s[-1] / 1e6 - 1) < 1e-6
    assert B.shape == (200, 2)


def test_growth_matrix_grows_under_partial_pivoting(pkg):
    n = 30
    A, _ = pkg.workloads.growth_matrix(n, 1)
    lu, piv, info = lapack.dgetrf(A)
    assert info == 0
    assert np.array_equal(piv, np.arange(n))  # no interchanges: the classic construction
    assert np.abs(np.triu(lu)).max() / np.abs(A).max() == 2.0 ** (n - 1)


def test_batch_sizes_and_offsets(pkg):
    w = pkg.workloads
    sizes, A, b, gam = w.batch(300, seed=3)
    assert sizes.min() >= 8 and sizes.max() <= 256 and len(sizes) == 300
    assert A.size == int((sizes ** 2).sum()) and b.size == int(sizes.sum())
    a_off, b_off = w.offsets(sizes)
    assert a_off[0] == 0 and b_off[0] == 0
    assert np.array_equal(np.diff(a_off), sizes[:-1] ** 2) and np.array_equal(np.diff(b_off), sizes[:-1])
    for i in (0, 17, 299):  # system i = I - g_i J_i, column-major at its offset
        n = int(sizes[i])
        Ai = A[a_off[i]:a_off[i] + n * n].reshape(n, n, order="F")
        J = (np.eye(n) - Ai) / gam[i]
        assert abs(np.linalg.norm(J) / np.sqrt(n) - 1) < 0.2  # J iid N(0, 1/n): ||J||_F ~ sqrt(n)
    s2 = w.batch(300, seed=3)
    assert all(np.array_equal(x, y) for x, y in zip((sizes, A, b, gam), s2))
