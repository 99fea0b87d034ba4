"""Seeded synthetic inputs with the shapes and distributions of the
benchmark configurations (no dataset is involved; every array is generated
from numpy's default_rng(seed), column-major FP64).

plain(n, nrhs)        A, B iid N(0,1)                       (n=1000 / n=8192 x 16 RHS)
shifted(n, nrhs)      A = G + 4 sqrt(n) I, G iid N(0,1)     (mixed precision, cond ~ 1e0-1e2)
svd_conditioned(n)    A = Q1 diag(s) Q2^T, s log-spaced 1..cond  (FP32-LU GMRES-IR case;
                      svd_conditioned_gpu builds the same on the GPU for large n)
growth_matrix(n)      Wilkinson's matrix, pivot growth 2^(n-1) under partial pivoting
batch(count)          A_i = I - g_i J_i, J_i iid N(0,1)/sqrt(n_i), n_i ~ U{8..256}, g_i ~ U[0.01,0.5]
"""
from __future__ import annotations

import numpy as np


def plain(n: int, nrhs: int = 1, seed: int = 0):
    rng = np.random.default_rng(seed)
    A = np.asfortranarray(rng.standard_normal((n, n)))
    B = np.asfortranarray(rng.standard_normal((n, nrhs)))
    return A, B


def shifted(n: int, nrhs: int = 1, seed: int = 0):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, n))
    A[np.diag_indices(n)] += 4.0 * np.sqrt(n)
    B = rng.standard_normal((n, nrhs))
    return np.asfortranarray(A), np.asfortranarray(B)


def svd_conditioned(n: int, nrhs: int = 1, cond: float = 1e6, seed: int = 0):
    """A = Q1 diag(sigma) Q2^T with sigma log-spaced in [1, cond] and Q1, Q2 the
    Q factors of seeded Gaussian matrices (numpy QR: use for n up to a few
    thousand on the host)."""
    rng = np.random.default_rng(seed)
    Q1, _ = np.linalg.qr(rng.standard_normal((n, n)))
    Q2, _ = np.linalg.qr(rng.standard_normal((n, n)))
    s = np.logspace(0.0, np.log10(cond), n)
    A = (Q1 * s) @ Q2.T
    B = rng.standard_normal((n, nrhs))
    return np.asfortranarray(A), np.asfortranarray(B)


def svd_conditioned_gpu(n: int, nrhs: int = 1, cond: float = 1e6, seed: int = 0):
    """svd_conditioned for large n: the same construction with the Gaussian
    matrices drawn from numpy default_rng(seed) and the two FP64 QR
    factorizations and the product done with torch on the current CUDA
    device (input generation only).  Returns host arrays, A column-major."""
    import torch
    rng = np.random.default_rng(seed)
    dev = torch.device("cuda", torch.cuda.current_device())
    s = torch.from_numpy(np.logspace(0.0, np.log10(cond), n)).to(dev)
    q1, _ = torch.linalg.qr(torch.from_numpy(rng.standard_normal((n, n))).to(dev))
    q2, _ = torch.linalg.qr(torch.from_numpy(rng.standard_normal((n, n))).to(dev))
    # A^T = Q2 diag(s) Q1^T in row-major order is A in column-major order
    at = (q2 * s) @ q1.T
    del q1, q2
    A = at.cpu().numpy().T
    del at
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    B = np.asfortranarray(rng.standard_normal((n, nrhs)))
    return A, B


def growth_matrix(n: int, nrhs: int = 1, seed: int = 0):
    """The classic worst case of partial pivoting (Wilkinson): 1 on the
    diagonal and in the last column, -1 below the diagonal.  No row
    interchange happens and the last column of U doubles at every step, so
    max|U| / max|A| = 2^(n-1)."""
    rng = np.random.default_rng(seed)
    A = -np.tril(np.ones((n, n)), -1) + np.eye(n)
    A[:, -1] = 1.0
    B = rng.standard_normal((n, nrhs))
    return np.asfortranarray(A), np.asfortranarray(B)


def batch(count: int, nmin: int = 8, nmax: int = 256, seed: int = 0):
    """Uneven batch: returns (sizes int64, A_packed, b_packed, gammas); system i
    is column-major n_i x n_i at offset sum_{k<i} n_k^2 of A_packed."""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(nmin, nmax + 1, size=count).astype(np.int64)
    gam = rng.uniform(0.01, 0.5, size=count)
    a_tot = int((sizes.astype(np.int64) ** 2).sum())
    A = np.empty(a_tot, dtype=np.float64)
    b = rng.standard_normal(int(sizes.sum()))
    off = 0
    for i, n in enumerate(sizes):
        n = int(n)
        J = rng.standard_normal((n, n)) / np.sqrt(n)
        Ai = -gam[i] * J
        Ai[np.diag_indices(n)] += 1.0
        A[off:off + n * n] = Ai.ravel(order="F")
        off += n * n
    return sizes, A, b, gam


def offsets(sizes: np.ndarray):
    sizes = np.asarray(sizes, dtype=np.int64)
    a_off = np.zeros(len(sizes), dtype=np.int64)
    b_off = np.zeros(len(sizes), dtype=np.int64)
    if len(sizes) > 1:
        a_off[1:] = np.cumsum(sizes[:-1] ** 2)
        b_off[1:] = np.cumsum(sizes[:-1])
    return a_off, b_off
