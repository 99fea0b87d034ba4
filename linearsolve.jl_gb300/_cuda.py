"""Minimal CUDA runtime plumbing over ctypes: device buffers and events.

Used to hold inputs resident in HBM and to time work on the library's
stream.  It loads the same libcudart.so.13 that libgblu.so links against.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_rt = None


def runtime() -> ctypes.CDLL:
    global _rt
    if _rt is None:
        from . import _lib
        _lib.load()  # libgblu pulls libcudart into the process first
        cands = ["libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so.13"]
        err = None
        for c in cands:
            try:
                _rt = ctypes.CDLL(c, mode=ctypes.RTLD_GLOBAL)
                break
            except OSError as e:  # pragma: no cover - depends on the image
                err = e
        if _rt is None:
            raise RuntimeError(f"cannot load libcudart: {err}")
        P, I = ctypes.c_void_p, ctypes.c_int
        _rt.cudaMalloc.argtypes = [ctypes.POINTER(P), ctypes.c_size_t]
        _rt.cudaFree.argtypes = [P]
        _rt.cudaMemcpy.argtypes = [P, P, ctypes.c_size_t, I]
        _rt.cudaMemcpyAsync.argtypes = [P, P, ctypes.c_size_t, I, P]
        _rt.cudaMemsetAsync.argtypes = [P, I, ctypes.c_size_t, P]
        _rt.cudaEventCreate.argtypes = [ctypes.POINTER(P)]
        _rt.cudaEventRecord.argtypes = [P, P]
        _rt.cudaEventSynchronize.argtypes = [P]
        _rt.cudaEventElapsedTime.argtypes = [ctypes.POINTER(ctypes.c_float), P, P]
        _rt.cudaEventDestroy.argtypes = [P]
        _rt.cudaStreamSynchronize.argtypes = [P]
        _rt.cudaDeviceSynchronize.argtypes = []
        _rt.cudaGetErrorString.restype = ctypes.c_char_p
        _rt.cudaGetErrorString.argtypes = [I]
        _rt.cudaHostAlloc.argtypes = [ctypes.POINTER(P), ctypes.c_size_t, ctypes.c_uint]
        _rt.cudaFreeHost.argtypes = [P]
    return _rt


def _ck(err: int, what: str) -> None:
    if err != 0:
        msg = runtime().cudaGetErrorString(err).decode()
        raise RuntimeError(f"{what}: {msg}")


H2D, D2H, D2D = 1, 2, 3


class DeviceMatrix:
    """A column-major float64 (or float32) matrix in device memory."""

    def __init__(self, rows: int, cols: int = 1, dtype=np.float64):
        self.rows, self.cols = int(rows), int(cols)
        self.dtype = np.dtype(dtype)
        self.ld = max(self.rows, 1)
        self.nbytes = self.ld * max(self.cols, 1) * self.dtype.itemsize
        p = ctypes.c_void_p()
        _ck(runtime().cudaMalloc(ctypes.byref(p), self.nbytes), "cudaMalloc")
        self.ptr = p.value

    @classmethod
    def from_host(cls, a: np.ndarray) -> "DeviceMatrix":
        a = np.asarray(a)
        a2 = a.reshape(a.shape[0], -1)
        dm = cls(a2.shape[0], a2.shape[1], a2.dtype)
        dm.upload(a2)
        return dm

    def upload(self, a: np.ndarray) -> None:
        a = np.asfortranarray(np.asarray(a, dtype=self.dtype).reshape(self.rows, self.cols))
        _ck(runtime().cudaMemcpy(self.ptr, a.ctypes.data, a.nbytes, H2D), "cudaMemcpy H2D")

    def to_host(self) -> np.ndarray:
        out = np.empty((self.rows, self.cols), dtype=self.dtype, order="F")
        _ck(runtime().cudaMemcpy(out.ctypes.data, self.ptr, out.nbytes, D2H), "cudaMemcpy D2H")
        return out

    def copy_from(self, other: "DeviceMatrix", stream=None) -> None:
        _ck(runtime().cudaMemcpyAsync(self.ptr, other.ptr, min(self.nbytes, other.nbytes), D2D,
                                      stream), "cudaMemcpyAsync D2D")

    def free(self) -> None:
        if self.ptr and getattr(self, "_owner", True):
            runtime().cudaFree(self.ptr)
        self.ptr = None

    def view(self, col0: int, ncols: int = 1) -> "DeviceMatrix":
        """Non-owning view of columns [col0, col0 + ncols)."""
        v = DeviceMatrix.__new__(DeviceMatrix)
        v.rows, v.cols, v.dtype, v.ld = self.rows, int(ncols), self.dtype, self.ld
        v.nbytes = v.ld * v.cols * v.dtype.itemsize
        v.ptr = self.ptr + col0 * self.ld * self.dtype.itemsize
        v._owner = False
        v._base = self
        return v


    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.free()
        except Exception:
            pass


def DeviceColumn(m: DeviceMatrix, j: int) -> DeviceMatrix:
    return m.view(j, 1)


class Event:
    def __init__(self):
        p = ctypes.c_void_p()
        _ck(runtime().cudaEventCreate(ctypes.byref(p)), "cudaEventCreate")
        self.ev = p.value

    def record(self, stream) -> None:
        _ck(runtime().cudaEventRecord(self.ev, stream), "cudaEventRecord")

    def synchronize(self) -> None:
        _ck(runtime().cudaEventSynchronize(self.ev), "cudaEventSynchronize")

    def elapsed_ms(self, end: "Event") -> float:
        ms = ctypes.c_float()
        _ck(runtime().cudaEventElapsedTime(ctypes.byref(ms), self.ev, end.ev), "cudaEventElapsedTime")
        return float(ms.value)


class PinnedArray:
    """Page-locked host memory viewed as a numpy array (for timed H2D/D2H)."""

    def __init__(self, shape, dtype=np.float64):
        self.dtype = np.dtype(dtype)
        n = int(np.prod(shape)) * self.dtype.itemsize
        p = ctypes.c_void_p()
        _ck(runtime().cudaHostAlloc(ctypes.byref(p), max(n, 1), 0), "cudaHostAlloc")
        self.ptr = p.value
        buf = (ctypes.c_char * max(n, 1)).from_address(self.ptr)
        self.array = np.frombuffer(buf, dtype=self.dtype, count=int(np.prod(shape))).reshape(
            shape, order="F")

    def free(self) -> None:
        if self.ptr:
            runtime().cudaFreeHost(self.ptr)
            self.ptr = None


def device_synchronize() -> None:
    _ck(runtime().cudaDeviceSynchronize(), "cudaDeviceSynchronize")
