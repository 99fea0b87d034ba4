"""CPU oracle for the dense LU path -- TEST INFRASTRUCTURE ONLY.

Only the test-suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package, and only as the checker (or, for the
benchmark, as the reported CPU baseline).  The GPU library never calls it.

Contents
--------
``lu_oracle.c``
    A plain-C restatement of LinearSolve.jl's in-tree blocked getrf
    (src/blocked_lufact.jl:38-743) and of its pure-Julia back-solve
    (src/factorization.jl:433-491), in the same fused-multiply-add order.
``oracle.py``
    ctypes bindings of that C file; the LAPACK stand-in
    (``scipy.linalg.lapack.dgetrf/dgetrs``, OpenBLAS, the library that
    ``LUFactorization`` reaches through ``LinearAlgebra.lu!``,
    src/factorization.jl:632-636,748); and the accuracy metrics.

Pinning: the C restatement is checked against the known answers and the
backward-stability metric of the reference's own tests
(test/Core/resolve.jl:78-106, test/Core/blocked_lufact.jl:11-28) and against
LAPACK's getrf (identical ipiv and factors within rounding) in tests/.
"""
from .oracle import *  # noqa: F401,F403
