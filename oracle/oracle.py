"""ctypes bindings of the C restatement, the LAPACK stand-in and the metrics.

TEST INFRASTRUCTURE ONLY (see the package docstring).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "lu_oracle.c")
_BUILD = os.path.join(_HERE, "_build")
_SO = os.path.join(_BUILD, "liblu_oracle.so")
_lock = threading.Lock()
_lib = None

__all__ = [
    "build", "lib", "getrf", "getrs", "getrf_nb", "gesv_batched",
    "lapack_getrf", "lapack_getrs", "lapack_solve",
    "backward_error", "forward_error", "scaled_residual", "luflop", "lu_flops",
    "apply_ipiv", "perm_from_ipiv",
]


def build(force: bool = False) -> str:
    """Compile lu_oracle.c with gcc into oracle/_build (no fp contraction:
    the FMAs the restatement needs are explicit fma() calls)."""
    os.makedirs(_BUILD, exist_ok=True)
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(_SRC):
        tmp = _SO + f".{os.getpid()}.tmp"
        subprocess.check_call([
            "gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-ffp-contract=off",
            "-fno-fast-math", "-o", tmp, _SRC, "-lm"])
        os.replace(tmp, _SO)
    return _SO


def lib() -> ctypes.CDLL:
    global _lib
    with _lock:
        if _lib is None:
            L = ctypes.CDLL(build())
            i64, p = ctypes.c_int64, ctypes.c_void_p
            for name in ("ora_dgetrf", "ora_sgetrf"):
                f = getattr(L, name)
                f.argtypes = [i64, i64, p, i64, p]
                f.restype = i64
            for name in ("ora_d_getrf_nb", "ora_s_getrf_nb"):
                f = getattr(L, name)
                f.argtypes = [i64, i64, p, i64, p, i64]
                f.restype = i64
            for name in ("ora_dgetrs", "ora_sgetrs"):
                f = getattr(L, name)
                f.argtypes = [ctypes.c_char, i64, i64, p, i64, p, p, i64]
                f.restype = None
            L.ora_dgesv_batched.argtypes = [i64, p, p, p, p, p, p, p]
            L.ora_dgesv_batched.restype = None
            _lib = L
    return _lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def getrf(A: np.ndarray):
    """Restated blocked getrf (blocked_lufact.jl:715-743).  Returns
    (LU column-major copy, ipiv int64 1-based, info)."""
    A = np.asarray(A)
    dt = np.float32 if A.dtype == np.float32 else np.float64
    LU = np.array(A, dtype=dt, order="F", copy=True)
    m, n = LU.shape
    ipiv = np.zeros(max(min(m, n), 1), dtype=np.int64)
    f = lib().ora_sgetrf if dt == np.float32 else lib().ora_dgetrf
    info = f(m, n, _ptr(LU), max(m, 1), _ptr(ipiv))
    return LU, ipiv[: min(m, n)], int(info)


def getrf_nb(A: np.ndarray, nb: int):
    """The blocked driver (blocked_lufact.jl:658-679) with an explicit panel width."""
    A = np.asarray(A)
    dt = np.float32 if A.dtype == np.float32 else np.float64
    LU = np.array(A, dtype=dt, order="F", copy=True)
    m, n = LU.shape
    ipiv = np.zeros(max(min(m, n), 1), dtype=np.int64)
    f = lib().ora_s_getrf_nb if dt == np.float32 else lib().ora_d_getrf_nb
    info = f(m, n, _ptr(LU), max(m, 1), _ptr(ipiv), nb)
    return LU, ipiv[: min(m, n)], int(info)


def getrs(LU: np.ndarray, ipiv: np.ndarray, B: np.ndarray, trans: str = "N"):
    """Restated back-solve (factorization.jl:433-457 per column; 'T' as LAPACK)."""
    dt = LU.dtype
    LU = np.asfortranarray(LU)
    ipiv = np.ascontiguousarray(ipiv, dtype=np.int64)
    vec = B.ndim == 1
    X = np.array(B.reshape(B.shape[0], -1), dtype=dt, order="F", copy=True)
    n = LU.shape[0]
    f = lib().ora_sgetrs if dt == np.float32 else lib().ora_dgetrs
    f(trans.encode(), n, X.shape[1], _ptr(LU), max(n, 1), _ptr(ipiv), _ptr(X), max(n, 1))
    return X[:, 0].copy() if vec else X


def gesv_batched(sizes, A_packed: np.ndarray, B_packed: np.ndarray):
    """Loop of restated getrf+getrs over back-to-back column-major systems."""
    sizes = np.ascontiguousarray(sizes, dtype=np.int64)
    a_off = np.zeros(len(sizes), dtype=np.int64)
    b_off = np.zeros(len(sizes), dtype=np.int64)
    if len(sizes) > 1:
        a_off[1:] = np.cumsum(sizes[:-1] ** 2)
        b_off[1:] = np.cumsum(sizes[:-1])
    A = np.array(A_packed, dtype=np.float64, copy=True)
    X = np.array(B_packed, dtype=np.float64, copy=True)
    work = np.zeros(int(sizes.max()) if len(sizes) else 1, dtype=np.int64)
    info = np.zeros(len(sizes), dtype=np.int64)
    lib().ora_dgesv_batched(len(sizes), _ptr(sizes), _ptr(a_off), _ptr(b_off),
                            _ptr(A), _ptr(X), _ptr(work), _ptr(info))
    return A, X, info


# --- LAPACK stand-in: the library LUFactorization calls -------------------

def lapack_getrf(A: np.ndarray):
    """scipy's dgetrf/sgetrf (OpenBLAS).  LUFactorization reaches the same
    routine through LinearAlgebra.lu! -> LAPACK.getrf! (factorization.jl:748).
    Returns (LU, ipiv int64 1-based, info)."""
    from scipy.linalg import lapack
    A = np.asarray(A)
    f = lapack.sgetrf if A.dtype == np.float32 else lapack.dgetrf
    lu, piv, info = f(A, overwrite_a=False)
    return np.asfortranarray(lu), piv.astype(np.int64) + 1, int(info)


def lapack_getrs(LU, ipiv, B, trans: str = "N"):
    from scipy.linalg import lapack
    f = lapack.sgetrs if LU.dtype == np.float32 else lapack.dgetrs
    x, info = f(LU, np.asarray(ipiv, dtype=np.int64) - 1, B, trans={"N": 0, "T": 1, "C": 2}[trans])
    if info != 0:
        raise ValueError(f"getrs info={info}")
    return x


def lapack_solve(A, B):
    LU, ipiv, info = lapack_getrf(A)
    return lapack_getrs(LU, ipiv, B), info


# --- metrics ----------------------------------------------------------------

def backward_error(A: np.ndarray, X: np.ndarray, B: np.ndarray) -> float:
    """Normwise backward error ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf),
    computed in FP64 (max over RHS columns)."""
    A = np.asarray(A, dtype=np.float64)
    X2 = np.asarray(X, dtype=np.float64).reshape(A.shape[1], -1)
    B2 = np.asarray(B, dtype=np.float64).reshape(A.shape[0], -1)
    R = B2 - A @ X2
    nA = np.abs(A).sum(axis=1).max() if A.size else 0.0
    worst = 0.0
    for c in range(X2.shape[1]):
        den = nA * np.abs(X2[:, c]).max(initial=0.0) + np.abs(B2[:, c]).max(initial=0.0)
        num = np.abs(R[:, c]).max(initial=0.0)
        worst = max(worst, (num / den) if den > 0 else (0.0 if num == 0 else np.inf))
    return float(worst)


def forward_error(X: np.ndarray, Xref: np.ndarray) -> float:
    X = np.asarray(X, dtype=np.float64)
    Xref = np.asarray(Xref, dtype=np.float64)
    den = np.abs(Xref).max(initial=0.0)
    return float(np.abs(X - Xref).max(initial=0.0) / den) if den > 0 else float(np.abs(X).max(initial=0.0))


def apply_ipiv(A: np.ndarray, ipiv: np.ndarray) -> np.ndarray:
    """P*A: the LAPACK interchange sequence applied to the rows of A."""
    PA = np.array(A, copy=True)
    for k, p in enumerate(np.asarray(ipiv) - 1):
        if p != k:
            PA[[k, p]] = PA[[p, k]]
    return PA


def perm_from_ipiv(ipiv: np.ndarray, m: int) -> np.ndarray:
    """perm with (P*A)[i] = A[perm[i]]."""
    perm = np.arange(m)
    for k, p in enumerate(np.asarray(ipiv) - 1):
        if p != k:
            perm[[k, p]] = perm[[p, k]]
    return perm


def scaled_residual(A: np.ndarray, LU: np.ndarray, ipiv: np.ndarray) -> float:
    """||P A - L U||_1 / (||L||_1 ||U||_1 eps max(m,n)), the backward-stability
    metric of test/Core/blocked_lufact.jl:11-28 (the reference requires < 20)."""
    A = np.asarray(A)
    dt = A.dtype if A.dtype in (np.float32, np.float64) else np.float64
    m, n = A.shape
    k = min(m, n)
    L = np.tril(LU[:, :k].astype(np.float64), -1)
    L[np.arange(k), np.arange(k)] = 1.0
    U = np.triu(LU[:k, :].astype(np.float64))
    PA = apply_ipiv(A.astype(np.float64), ipiv)
    eps = float(np.finfo(dt).eps)
    den = np.linalg.norm(L, 1) * np.linalg.norm(U, 1) * eps * max(m, n)
    return float(np.linalg.norm(PA - L @ U, 1) / den) if den > 0 else 0.0


def luflop(m: int, n: int | None = None) -> float:
    """The reference benchmark's flop count, computed exactly as benchmarks/lu.jl:8-20
    (= lib/LinearSolveAutotune/src/algorithms.jl:146-159) computes it.  Note that
    its ``scaleflop`` term is ``sum((k+1):m)``, the SUM of the row indices, not
    their count; this function keeps that so GFLOP/s figures are comparable."""
    n = m if n is None else n
    total = 0
    for k in range(1, min(m, n) + 1):
        scale = (m * (m + 1) - k * (k + 1)) // 2 if k < m else 0
        total += 1 + scale + 2 * (m - k) * (n - k)
    return float(total)


def lu_flops(m: int, n: int | None = None) -> float:
    """Arithmetic flop count of partial-pivot LU: sum_k [1 + (m-k) + 2 (m-k)(n-k)]
    (one reciprocal, m-k scalings, (m-k)(n-k) fused multiply-adds), ~2n^3/3."""
    n = m if n is None else n
    total = 0
    for k in range(1, min(m, n) + 1):
        total += 1 + (m - k) + 2 * (m - k) * (n - k)
    return float(total)
