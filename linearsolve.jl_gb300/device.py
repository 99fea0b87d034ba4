"""Python handles over the C ABI: a context (device + stream + HBM budget) and
device-resident factorizations.  This is the layer LinearCache drives; it is
the Python twin of the Julia binding in julia/GB300LinearSolve.jl.
"""
from __future__ import annotations

import ctypes
import threading

import numpy as np

from . import _lib
from ._cuda import DeviceMatrix
from ._lib import GBLUError, RefineOpts, RefineStats, check

PRECISIONS = {"fp64": _lib.GBLU_FP64, "fp32": _lib.GBLU_FP32, "bf16": _lib.GBLU_BF16,
              "fp16": _lib.GBLU_FP16}
REFINE_MODES = {"ir": _lib.GBLU_REFINE_IR, "gmres_ir": _lib.GBLU_REFINE_GMRES}


class Context:
    """One device, one stream, one HBM budget (gblu_create)."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0):
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        st = self.lib.gblu_create(ctypes.byref(h), int(device), int(hbm_budget_bytes))
        check(st, None)
        self.handle = h
        self.device = device

    @property
    def stream(self) -> int:
        s = ctypes.c_void_p()
        check(self.lib.gblu_ctx_stream(self.handle, ctypes.byref(s)), self.handle)
        return s.value or 0

    def memory(self) -> tuple[int, int]:
        a, b = ctypes.c_uint64(), ctypes.c_uint64()
        check(self.lib.gblu_ctx_memory(self.handle, ctypes.byref(a), ctypes.byref(b)), self.handle)
        return a.value, b.value

    def profile_enable(self, enable: bool = True) -> None:
        check(self.lib.gblu_profile_enable(self.handle, 1 if enable else 0), self.handle)

    def profile_read(self, reset: bool = False) -> dict:
        """Launch counts, event-timed ms, flops and bytes per kernel kind."""
        pr = _lib.Profile()
        check(self.lib.gblu_profile_read(self.handle, ctypes.byref(pr), 1 if reset else 0),
              self.handle)
        out = {"launches": int(pr.launches)}
        for i, name in enumerate(_lib.KIND_NAMES):
            out[name] = {"count": int(pr.count[i]), "ms": float(pr.ms[i]),
                         "flops": float(pr.flops[i]), "bytes": float(pr.bytes[i])}
        return out

    def gemm_update(self, C: np.ndarray, A: np.ndarray, B: np.ndarray, precision: str = "bf16"):
        """C - A @ B with the getrf trailing-update kernel (host arrays, FP32)."""
        Cf = np.array(C, dtype=np.float32, order="F", copy=True)
        Af = np.asfortranarray(np.asarray(A, dtype=np.float32))
        Bf = np.asfortranarray(np.asarray(B, dtype=np.float32))
        m, k = Af.shape
        n = Bf.shape[1]
        check(self.lib.gblu_gemm_update(self.handle, PRECISIONS[precision], m, n, k, Af.ctypes.data,
                                        max(m, 1), Bf.ctypes.data, max(k, 1), Cf.ctypes.data,
                                        max(m, 1), _lib.GBLU_HOST), self.handle)
        return Cf

    def factor(self, m: int, n: int | None = None, precision: str = "fp64") -> "Factorization":
        return Factorization(self, m, m if n is None else n, precision)

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.gblu_destroy(self.handle)
            self.handle = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


_default_ctx: dict[int, Context] = {}
_default_lock = threading.Lock()


def default_context(device: int = 0) -> Context:
    with _default_lock:
        ctx = _default_ctx.get(device)
        if ctx is None:
            ctx = Context(device)
            _default_ctx[device] = ctx
        return ctx


def _as_fortran(a: np.ndarray, dtype=np.float64) -> np.ndarray:
    return np.asfortranarray(np.asarray(a, dtype=dtype))


class Factorization:
    """A gblu_factor: factors + ipiv + scratch resident in HBM."""

    def __init__(self, ctx: Context, m: int, n: int, precision: str = "fp64"):
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(PRECISIONS)}")
        self.ctx, self.lib = ctx, ctx.lib
        self.m, self.n, self.precision = int(m), int(n), precision
        h = ctypes.c_void_p()
        check(self.lib.gblu_factor_create(ctx.handle, self.m, self.n, PRECISIONS[precision],
                                          ctypes.byref(h)), ctx.handle)
        self.handle = h
        self.info = None

    # -- getrf ---------------------------------------------------------------
    def getrf(self, A) -> int:
        """Factor A (numpy array or DeviceMatrix).  Returns LAPACK info."""
        info = ctypes.c_int64()
        if isinstance(A, DeviceMatrix):
            if (A.rows, A.cols) != (self.m, self.n):
                raise ValueError("shape mismatch")
            st = self.lib.gblu_getrf(self.ctx.handle, self.handle, A.ptr, A.ld, _lib.GBLU_DEVICE,
                                     ctypes.byref(info))
        else:
            Af = _as_fortran(A)
            if Af.shape != (self.m, self.n):
                raise ValueError(f"A has shape {Af.shape}, factor is {(self.m, self.n)}")
            st = self.lib.gblu_getrf(self.ctx.handle, self.handle, Af.ctypes.data, max(self.m, 1),
                                     _lib.GBLU_HOST, ctypes.byref(info))
        check(st, self.ctx.handle)
        self.info = int(info.value)
        return self.info

    # -- getrs ---------------------------------------------------------------
    def getrs(self, B, trans: str = "N"):
        """Solve op(A) X = B.  numpy B: returns a new array; DeviceMatrix: in place."""
        if isinstance(B, DeviceMatrix):
            check(self.lib.gblu_getrs(self.ctx.handle, self.handle, trans.encode(), B.cols, B.ptr,
                                      B.ld, _lib.GBLU_DEVICE), self.ctx.handle)
            return B
        B = np.asarray(B, dtype=np.float64)
        vec = B.ndim == 1
        X = np.array(B.reshape(B.shape[0], -1), dtype=np.float64, order="F", copy=True)
        check(self.lib.gblu_getrs(self.ctx.handle, self.handle, trans.encode(), X.shape[1],
                                  X.ctypes.data, max(X.shape[0], 1), _lib.GBLU_HOST), self.ctx.handle)
        return X[:, 0].copy() if vec else X

    def solve_refined(self, B, trans: str = "N", mode: str = "ir", max_iter: int = 30,
                      tol: float = 0.0, fallback: bool = True, gmres_restart: int = 30,
                      gmres_tol: float = 1e-10, growth_limit: float = 0.0):
        """Refined solve; returns (X, stats dict)."""
        o = RefineOpts()
        check(self.lib.gblu_refine_opts_default(ctypes.byref(o)), None)
        o.mode = REFINE_MODES[mode]
        o.max_iter = int(max_iter)
        o.tol = float(tol)
        o.fallback = 1 if fallback else 0
        o.gmres_restart = int(gmres_restart)
        o.gmres_tol = float(gmres_tol)
        o.growth_limit = float(growth_limit)
        s = RefineStats()
        if isinstance(B, DeviceMatrix):
            check(self.lib.gblu_solve_refined(self.ctx.handle, self.handle, trans.encode(), B.cols,
                                              B.ptr, B.ld, _lib.GBLU_DEVICE, ctypes.byref(o),
                                              ctypes.byref(s)), self.ctx.handle)
            X = B
        else:
            B = np.asarray(B, dtype=np.float64)
            vec = B.ndim == 1
            X = np.array(B.reshape(B.shape[0], -1), dtype=np.float64, order="F", copy=True)
            check(self.lib.gblu_solve_refined(self.ctx.handle, self.handle, trans.encode(),
                                              X.shape[1], X.ctypes.data, max(X.shape[0], 1),
                                              _lib.GBLU_HOST, ctypes.byref(o), ctypes.byref(s)),
                  self.ctx.handle)
            X = X[:, 0].copy() if vec else X
        stats = {k: getattr(s, k) for k, _ in RefineStats._fields_ if k != "pad_"}
        return X, stats

    def set_solve(self, mode: str = "exact") -> None:
        """getrs mode: "exact" (the reference back-solve's per-row order,
        bit-identical) or "fast" (inverted 64 x 64 diagonal blocks; backward-
        error accurate).  For mixed factors: the low-precision solve inside
        refinement."""
        modes = {"exact": _lib.GBLU_SOLVE_EXACT, "fast": _lib.GBLU_SOLVE_FAST}
        if mode not in modes:
            raise ValueError("solve mode must be 'exact' or 'fast'")
        check(self.lib.gblu_factor_set_solve(self.ctx.handle, self.handle, modes[mode]), self.ctx.handle)
        self.solve_mode = mode

    def set_pivoting(self, mode: str = "partial") -> None:
        """Pivoting of a mixed factor's low-precision LU from the next getrf
        on: "partial" (default, the reference's order), "tournament" (CALU's
        tall-skinny panel for leaves over 512 rows) or "rbt" (no pivoting after
        a depth-2 random butterfly transform of both sides; n a multiple of
        4).  Changing it invalidates the current factors."""
        modes = {"partial": _lib.GBLU_PIVOT_PARTIAL, "tournament": _lib.GBLU_PIVOT_TOURNAMENT,
                 "rbt": _lib.GBLU_PIVOT_RBT}
        if mode not in modes:
            raise ValueError("pivoting must be 'partial', 'tournament' or 'rbt'")
        check(self.lib.gblu_factor_set_pivoting(self.ctx.handle, self.handle, modes[mode]), self.ctx.handle)
        self.pivoting = mode

    def keep_matrix(self, keep: bool = True) -> None:
        """FP64 factors: keep a device copy of A from the next getrf on, for
        residual_norm (mixed factors keep A anyway)."""
        check(self.lib.gblu_factor_keep_matrix(self.ctx.handle, self.handle, 1 if keep else 0),
              self.ctx.handle)

    def residual_norm(self, X, B, trans: str = "N") -> tuple[float, float]:
        """(||B - op(A) X||_F, ||B||_F) computed on the device with the kept A."""
        r, bn = ctypes.c_double(), ctypes.c_double()
        if isinstance(X, DeviceMatrix) and isinstance(B, DeviceMatrix):
            st = self.lib.gblu_residual_norm(self.ctx.handle, self.handle, trans.encode(), X.cols, X.ptr,
                                             X.ld, B.ptr, B.ld, _lib.GBLU_DEVICE, ctypes.byref(r),
                                             ctypes.byref(bn))
        else:
            X = X.to_host() if isinstance(X, DeviceMatrix) else X
            B = B.to_host() if isinstance(B, DeviceMatrix) else B
            Xf = np.asfortranarray(np.asarray(X, dtype=np.float64).reshape(self.n, -1))
            Bf = np.asfortranarray(np.asarray(B, dtype=np.float64).reshape(self.n, -1))
            st = self.lib.gblu_residual_norm(self.ctx.handle, self.handle, trans.encode(), Xf.shape[1],
                                             Xf.ctypes.data, max(self.n, 1), Bf.ctypes.data, max(self.n, 1),
                                             _lib.GBLU_HOST, ctypes.byref(r), ctypes.byref(bn))
        check(st, self.ctx.handle)
        return float(r.value), float(bn.value)

    def growth(self) -> float:
        """Pivot growth max|U| / max|A| of the last getrf (mixed precisions)."""
        g = ctypes.c_double()
        check(self.lib.gblu_get_growth(self.ctx.handle, self.handle, ctypes.byref(g)), self.ctx.handle)
        return float(g.value)

    # -- inspection ------------------------------------------------------------
    def ipiv(self) -> np.ndarray:
        out = np.zeros(max(min(self.m, self.n), 1), dtype=np.int64)
        check(self.lib.gblu_get_ipiv(self.ctx.handle, self.handle, out.ctypes.data), self.ctx.handle)
        return out[: min(self.m, self.n)]

    def factors(self) -> np.ndarray:
        out = np.zeros((self.m, self.n), dtype=np.float64, order="F")
        check(self.lib.gblu_get_factors(self.ctx.handle, self.handle, out.ctypes.data,
                                        max(self.m, 1)), self.ctx.handle)
        return out

    def close(self) -> None:
        if getattr(self, "handle", None) and self.ctx.handle:
            self.lib.gblu_factor_destroy(self.ctx.handle, self.handle)
        self.handle = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """A gblu_batch: `len(sizes)` independent square systems (n_i <= 256)
    packed back to back, solved by one graph launch (gblu_batch_*)."""

    def __init__(self, ctx: Context, sizes, precision: str = "fp64"):
        if precision not in ("fp64", "fp32"):
            raise ValueError("batched precision must be 'fp64' or 'fp32'")
        self.ctx, self.lib = ctx, ctx.lib
        self.sizes = np.ascontiguousarray(sizes, dtype=np.int64)
        h = ctypes.c_void_p()
        check(self.lib.gblu_batch_create(ctx.handle, len(self.sizes), self.sizes.ctypes.data,
                                         PRECISIONS[precision], ctypes.byref(h)), ctx.handle)
        self.handle = h
        self.info = np.zeros(len(self.sizes), dtype=np.int64)

    def solve(self, A, b):
        """Host arrays: A packed column-major systems, b packed right-hand
        sides; returns the packed solutions (new array).  DeviceMatrix
        arguments: solved in place of b."""
        if isinstance(A, DeviceMatrix):
            check(self.lib.gblu_batch_solve(self.ctx.handle, self.handle, A.ptr, b.ptr, _lib.GBLU_DEVICE,
                                            self.info.ctypes.data), self.ctx.handle)
            return b
        A = np.ascontiguousarray(A, dtype=np.float64)
        x = np.array(b, dtype=np.float64, copy=True)
        check(self.lib.gblu_batch_solve(self.ctx.handle, self.handle, A.ctypes.data, x.ctypes.data,
                                        _lib.GBLU_HOST, self.info.ctypes.data), self.ctx.handle)
        return x

    def iterations(self) -> np.ndarray:
        its = np.zeros(len(self.sizes), dtype=np.int32)
        check(self.lib.gblu_batch_iterations(self.ctx.handle, self.handle, its.ctypes.data), self.ctx.handle)
        return its

    def close(self) -> None:
        if getattr(self, "handle", None) and self.ctx.handle:
            self.lib.gblu_batch_destroy(self.ctx.handle, self.handle)
        self.handle = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass


# -- LAPACK-shaped convenience wrappers (host buffers, default context) -------

def dgetrf(A: np.ndarray):
    """gblu_dgetrf_: returns (LU, ipiv, info) like scipy.linalg.lapack.dgetrf
    but with 1-based int64 ipiv."""
    lib = _lib.load()
    LU = np.array(A, dtype=np.float64, order="F", copy=True)
    m, n = LU.shape
    ipiv = np.zeros(max(min(m, n), 1), dtype=np.int64)
    mm, nn, lda, info = ctypes.c_int64(m), ctypes.c_int64(n), ctypes.c_int64(max(m, 1)), ctypes.c_int64()
    lib.gblu_dgetrf_(ctypes.byref(mm), ctypes.byref(nn), LU.ctypes.data, ctypes.byref(lda),
                     ipiv.ctypes.data, ctypes.byref(info))
    if info.value <= -1000:
        raise GBLUError(int(-1000 - info.value), lib.gblu_last_error(None).decode())
    return LU, ipiv[: min(m, n)], int(info.value)


def dgetrs(LU: np.ndarray, ipiv: np.ndarray, B: np.ndarray, trans: str = "N"):
    lib = _lib.load()
    LU = _as_fortran(LU)
    ipiv = np.ascontiguousarray(ipiv, dtype=np.int64)
    vec = np.ndim(B) == 1
    X = np.array(np.asarray(B, dtype=np.float64).reshape(LU.shape[0], -1), order="F", copy=True)
    n, nrhs = ctypes.c_int64(LU.shape[0]), ctypes.c_int64(X.shape[1])
    lda, ldb, info = ctypes.c_int64(max(LU.shape[0], 1)), ctypes.c_int64(max(X.shape[0], 1)), ctypes.c_int64()
    lib.gblu_dgetrs_(trans.encode(), ctypes.byref(n), ctypes.byref(nrhs), LU.ctypes.data,
                     ctypes.byref(lda), ipiv.ctypes.data, X.ctypes.data, ctypes.byref(ldb),
                     ctypes.byref(info), 1)
    if info.value != 0:
        raise GBLUError(int(-1000 - info.value) if info.value <= -1000 else _lib.GBLU_EINVAL,
                        f"dgetrs info={info.value}: {lib.gblu_last_error(None).decode()}")
    return X[:, 0].copy() if vec else X
