"""The allocation-free solve (gblu_dgetrs_noalloc).

It exists for callers that must not allocate device memory during a solve:
per-step solver loops such as Newton iterations inside an ODE integrator,
where a cudaMalloc/cudaFree would synchronise the device; hosts whose device
memory is committed to a fixed budget.  Its scratch is a fixed array compiled
into the library instead of memory from an allocator.

The test calls it through the C ABI on device buffers the test owns and
compares it with the existing gblu_getrs on the same factors, twice in a row
(the shared scratch keeps the previous call's contents).  The getrs kernels
are bit-exact, so the comparison is exact.  This file is named to be
collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _free_device_bytes(cu):
    free, total = ctypes.c_size_t(), ctypes.c_size_t()
    rt = cu.runtime()
    rt.cudaMemGetInfo.argtypes = [ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)]
    assert rt.cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0
    return free.value


@pytest.mark.parametrize("n,nrhs", [(1, 1), (300, 3), (2049, 11)])
def test_noalloc_matches_getrs_twice(pkg, n, nrhs):
    from importlib import import_module
    cu = import_module(pkg.__name__ + "._cuda")
    lib = pkg.load_library()
    ctx = pkg.Context(0)
    rng = np.random.default_rng(4242 + n)
    A = rng.standard_normal((n, n))
    f = ctx.factor(n, n)
    assert f.getrf(A) == 0
    LU, ipiv = f.factors(), f.ipiv()
    dLU = pkg.DeviceMatrix.from_host(LU)
    dipiv = pkg.DeviceMatrix.from_host(ipiv.reshape(-1, 1).astype(np.int64))
    for call in range(2):
        for trans in ("N", "T"):
            B = rng.standard_normal((n, nrhs))
            X_ref = f.getrs(B, trans=trans)  # the existing entry point
            dB = pkg.DeviceMatrix.from_host(B)
            free_before = _free_device_bytes(cu)
            st = lib.gblu_dgetrs_noalloc(trans.encode(), n, nrhs, dLU.ptr, n, dipiv.ptr, dB.ptr,
                                         n, None)
            if call == 1 or trans == "T":  # every call after the first
                assert _free_device_bytes(cu) == free_before  # nothing was allocated
            assert st == 0, lib.gblu_last_error(None)
            assert np.array_equal(dB.to_host(), X_ref), (call, trans)
            dB.free()
    f.close()
    ctx.close()


def test_noalloc_rejects_sizes_beyond_limit(pkg):
    lib = pkg.load_library()
    st = lib.gblu_dgetrs_noalloc(b"N", 16385, 1, None, 16385, None, None, 16385, None)
    assert st == 7  # GBLU_EUNSUPPORTED, before touching any device memory
    assert b"16384" in lib.gblu_last_error(None)


def test_noalloc_reports_invalid_pivot(pkg):
    """An out-of-range pivot is found on the device (the permutation kernel
    checks every pivot against [k, n) and stops): GBLU_EINVAL, and the next
    call with valid pivots is correct again."""
    lib = pkg.load_library()
    ctx = pkg.Context(0)
    n = 200
    rng = np.random.default_rng(77)
    A = rng.standard_normal((n, n))
    f = ctx.factor(n, n)
    assert f.getrf(A) == 0
    LU, ipiv = f.factors(), f.ipiv()
    dLU = pkg.DeviceMatrix.from_host(LU)
    bad = ipiv.copy()
    bad[17] = n + 5  # beyond the matrix
    dbad = pkg.DeviceMatrix.from_host(bad.reshape(-1, 1).astype(np.int64))
    B = rng.standard_normal((n, 2))
    dB = pkg.DeviceMatrix.from_host(B)
    st = lib.gblu_dgetrs_noalloc(b"N", n, 2, dLU.ptr, n, dbad.ptr, dB.ptr, n, None)
    assert st == 1, lib.gblu_last_error(None)  # GBLU_EINVAL
    assert b"ipiv" in lib.gblu_last_error(None)
    dgood = pkg.DeviceMatrix.from_host(ipiv.reshape(-1, 1).astype(np.int64))
    dB2 = pkg.DeviceMatrix.from_host(B)
    assert lib.gblu_dgetrs_noalloc(b"N", n, 2, dLU.ptr, n, dgood.ptr, dB2.ptr, n, None) == 0
    assert np.array_equal(dB2.to_host(), f.getrs(B))
    for d in (dLU, dbad, dB, dgood, dB2):
        d.free()
    f.close()
    ctx.close()
