"""Failure detection without a GPU fault: every spin-wait in the kernels
(the cooperative panel's grid barrier, getrs value polling, the register
panel's mbarrier wait) reads %globaltimer and gives up after its limit with
a DEV_* code in the scratch error word.  Each test makes one wait run out on
a count, value or phase that nothing provides, checks the code, and then
checks that the same context still factors bit-exactly."""
import ctypes
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DEV_TIMEOUT_PANEL = 1
DEV_TIMEOUT_SOLVE = 2


def _tools():
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    lib = ctypes.CDLL(os.path.join(root, "linearsolve.jl_gb300", "libgblu_tools.so"))
    lib.gblu_tool_waitcheck.argtypes = [ctypes.c_int32, ctypes.POINTER(ctypes.c_int32),
                                        ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_double)]
    lib.gblu_tool_waitcheck.restype = ctypes.c_int32
    return lib


@pytest.mark.parametrize("which,expected", [(0, DEV_TIMEOUT_PANEL), (1, DEV_TIMEOUT_SOLVE),
                                            (2, DEV_TIMEOUT_PANEL)],
                         ids=["grid-barrier", "getrs-poll", "panel-mbarrier"])
def test_bounded_wait_gives_up(ctx, oracle_mod, which, expected):
    lib = _tools()
    code, gave_up, secs = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_double()
    assert lib.gblu_tool_waitcheck(which, ctypes.byref(code), ctypes.byref(gave_up), ctypes.byref(secs)) == 0
    assert gave_up.value == 1
    assert code.value == expected
    assert 1.0 < secs.value < 30.0, secs.value  # the 2 s limit, not a hang
    # the context is still usable: a factorization right after is bit-exact
    rng = np.random.default_rng(which)
    A = rng.standard_normal((300, 300))
    f = ctx.factor(300, 300)
    assert f.getrf(A) == 0
    LU, ipiv, _ = oracle_mod.getrf(A)
    assert np.array_equal(f.factors(), LU)
    assert np.array_equal(f.ipiv(), ipiv)
    f.close()
