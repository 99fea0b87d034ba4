"""ctypes binding of libgblu.so (include/gblu.h).

The library is loaded from this package directory.  There is no fallback: if
the shared object is missing or cannot be loaded, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgblu.so")

# status codes (gblu.h)
GBLU_OK = 0
GBLU_EINVAL = 1
GBLU_ECUDA = 2
GBLU_ENOMEM = 3
GBLU_ETIMEOUT = 4
GBLU_ENOTFACTORED = 5
GBLU_ESTALL = 6
GBLU_EUNSUPPORTED = 7
GBLU_ENODEVICE = 8

GBLU_FP64 = 0
GBLU_FP32 = 1
GBLU_BF16 = 2
GBLU_FP16 = 3

GBLU_HOST = 0
GBLU_DEVICE = 1

GBLU_REFINE_IR = 0
GBLU_REFINE_GMRES = 1

GBLU_SOLVE_EXACT = 0
GBLU_SOLVE_FAST = 1
GBLU_PIVOT_PARTIAL = 0
GBLU_PIVOT_TOURNAMENT = 1
GBLU_PIVOT_RBT = 2

STATUS_NAMES = {
    0: "GBLU_OK", 1: "GBLU_EINVAL", 2: "GBLU_ECUDA", 3: "GBLU_ENOMEM", 4: "GBLU_ETIMEOUT",
    5: "GBLU_ENOTFACTORED", 6: "GBLU_ESTALL", 7: "GBLU_EUNSUPPORTED", 8: "GBLU_ENODEVICE",
}


class GBLUError(RuntimeError):
    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


class RefineOpts(ctypes.Structure):
    _fields_ = [
        ("mode", ctypes.c_int32), ("max_iter", ctypes.c_int32), ("tol", ctypes.c_double),
        ("fallback", ctypes.c_int32), ("gmres_restart", ctypes.c_int32),
        ("gmres_tol", ctypes.c_double), ("growth_limit", ctypes.c_double),
    ]


GBLU_FALLBACK_NONE = 0
GBLU_FALLBACK_STALL = 1
GBLU_FALLBACK_GROWTH = 2
GBLU_FALLBACK_ZERO_PIVOT = 3


class RefineStats(ctypes.Structure):
    _fields_ = [
        ("iterations", ctypes.c_int32), ("inner_iterations", ctypes.c_int32),
        ("converged", ctypes.c_int32), ("fell_back", ctypes.c_int32),
        ("backward_error", ctypes.c_double), ("growth", ctypes.c_double),
        ("fallback_reason", ctypes.c_int32), ("pad_", ctypes.c_int32),
    ]


PROFILE_KINDS = 9
KIND_NAMES = ["gemm", "panel", "laswp", "trsm", "perm", "getrs", "refine", "batched", "other"]


class Profile(ctypes.Structure):
    _fields_ = [
        ("launches", ctypes.c_uint64),
        ("count", ctypes.c_uint64 * PROFILE_KINDS),
        ("ms", ctypes.c_double * PROFILE_KINDS),
        ("flops", ctypes.c_double * PROFILE_KINDS),
        ("bytes", ctypes.c_double * PROFILE_KINDS),
    ]


class ServeConfig(ctypes.Structure):
    _fields_ = [("workers", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("refine_mode", ctypes.c_int32), ("hbm_budget_bytes", ctypes.c_uint64),
                ("max_rhs_batch", ctypes.c_int32), ("small_n", ctypes.c_int32),
                ("solve_mode", ctypes.c_int32), ("max_small_batch", ctypes.c_int32),
                ("large_n", ctypes.c_int32), ("max_large", ctypes.c_int32),
                ("pivoting", ctypes.c_int32)]


class Request(ctypes.Structure):
    _fields_ = [("key", ctypes.c_uint64), ("n", ctypes.c_int64), ("A", ctypes.c_void_p),
                ("b", ctypes.c_void_p), ("x", ctypes.c_void_p), ("tag", ctypes.c_uint64)]


class Completion(ctypes.Structure):
    _fields_ = [("tag", ctypes.c_uint64), ("status", ctypes.c_int32), ("refactored", ctypes.c_int32),
                ("fell_back", ctypes.c_int32), ("iterations", ctypes.c_int32),
                ("info", ctypes.c_int64), ("backward_error", ctypes.c_double),
                ("latency_us", ctypes.c_double), ("queue_us", ctypes.c_double)]


class ServeStats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int64) for k in (
        "submitted", "completed", "failed", "factorizations", "solves", "merged_solves",
        "evictions", "resident_factors", "queued", "in_flight")] + [("resident_bytes", ctypes.c_uint64)] + [
        (k, ctypes.c_int64) for k in ("small_launches", "small_systems", "admission_waits")]


_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_U64 = ctypes.c_uint64
_PI64 = ctypes.POINTER(ctypes.c_int64)

# name -> (restype, argtypes): every function include/gblu.h declares
SIGNATURES = {
    "gblu_version": (_I32, []),
    "gblu_create": (_I32, [ctypes.POINTER(_P), _I32, _U64]),
    "gblu_destroy": (_I32, [_P]),
    "gblu_last_error": (ctypes.c_char_p, [_P]),
    "gblu_ctx_stream": (_I32, [_P, ctypes.POINTER(_P)]),
    "gblu_ctx_memory": (_I32, [_P, ctypes.POINTER(_U64), ctypes.POINTER(_U64)]),
    "gblu_profile_enable": (_I32, [_P, _I32]),
    "gblu_profile_read": (_I32, [_P, ctypes.POINTER(Profile), _I32]),
    "gblu_factor_create": (_I32, [_P, _I64, _I64, _I32, ctypes.POINTER(_P)]),
    "gblu_factor_destroy": (_I32, [_P, _P]),
    "gblu_getrf": (_I32, [_P, _P, _P, _I64, _I32, _PI64]),
    "gblu_getrs": (_I32, [_P, _P, ctypes.c_char, _I64, _P, _I64, _I32]),
    "gblu_gemm_update": (_I32, [_P, _I32, _I64, _I64, _I64, _P, _I64, _P, _I64, _P, _I64, _I32]),
    "gblu_get_ipiv": (_I32, [_P, _P, _P]),
    "gblu_get_factors": (_I32, [_P, _P, _P, _I64]),
    "gblu_get_info": (_I32, [_P, _P, _PI64]),
    "gblu_get_growth": (_I32, [_P, _P, ctypes.POINTER(ctypes.c_double)]),
    "gblu_factor_keep_matrix": (_I32, [_P, _P, _I32]),
    "gblu_factor_set_solve": (_I32, [_P, _P, _I32]),
    "gblu_factor_set_pivoting": (_I32, [_P, _P, _I32]),
    "gblu_residual_norm": (_I32, [_P, _P, ctypes.c_char, _I64, _P, _I64, _P, _I64, _I32,
                                  ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "gblu_refine_opts_default": (_I32, [ctypes.POINTER(RefineOpts)]),
    "gblu_solve_refined": (_I32, [_P, _P, ctypes.c_char, _I64, _P, _I64, _I32,
                                  ctypes.POINTER(RefineOpts), ctypes.POINTER(RefineStats)]),
    "gblu_batch_create": (_I32, [_P, _I64, _P, _I32, ctypes.POINTER(_P)]),
    "gblu_batch_schedule": (_I32, [_P, _P, _I32, _P, _P, _P, _P]),
    "gblu_batch_solve": (_I32, [_P, _P, _P, _P, _I32, _P]),
    "gblu_batch_iterations": (_I32, [_P, _P, _P]),
    "gblu_batch_destroy": (_I32, [_P, _P]),
    "gblu_serve_config_default": (_I32, [ctypes.POINTER(ServeConfig)]),
    "gblu_serve_create": (_I32, [_P, ctypes.POINTER(ServeConfig), ctypes.POINTER(_P)]),
    "gblu_serve_submit": (_I32, [_P, ctypes.POINTER(Request)]),
    "gblu_serve_poll": (_I32, [_P, ctypes.POINTER(Completion), _I32, ctypes.POINTER(_I32), _I32]),
    "gblu_serve_get_stats": (_I32, [_P, ctypes.POINTER(ServeStats)]),
    "gblu_serve_destroy": (_I32, [_P]),
    "gblu_dgetrs_noalloc": (_I32, [ctypes.c_char, _I64, _I64, _P, _I64, _P, _P, _I64, _P]),
    "gblu_dgetrf_": (None, [_PI64, _PI64, _P, _PI64, _P, _PI64]),
    "gblu_dgetrs_": (None, [ctypes.c_char_p, _PI64, _PI64, _P, _PI64, _P, _P, _PI64, _PI64,
                            ctypes.c_long]),
    "gblu_sgetrf_": (None, [_PI64, _PI64, _P, _PI64, _P, _PI64]),
    "gblu_sgetrs_": (None, [ctypes.c_char_p, _PI64, _PI64, _P, _PI64, _P, _P, _PI64, _PI64,
                            ctypes.c_long]),
}

_lock = threading.Lock()
_lib = None


def load() -> ctypes.CDLL:
    """Load libgblu.so (building it first if the sources are newer)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise GBLUError(GBLU_ENODEVICE,
                            f"{LIB_PATH} is missing; run __graft_entry__.build() first")
        lib = ctypes.CDLL(LIB_PATH, mode=ctypes.RTLD_GLOBAL)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(status: int, ctx=None) -> None:
    if status != GBLU_OK:
        lib = load()
        msg = lib.gblu_last_error(ctx)
        raise GBLUError(status, (msg or b"").decode(errors="replace"))
