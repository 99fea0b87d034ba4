"""GB300-native dense LU for LinearSolve.jl's LU path.

The compute lives in ``libgblu.so`` (CUDA for sm_103a, C ABI declared in
``include/gblu.h``).  This package is its Python host side:

``linear``    LinearProblem / init / solve / solve! (``solve_bang``) / LinearCache
              and the algorithm types GB300LUFactorization and
              GB300MixedLUFactorization, mirroring LinearSolve.jl's interface.
``device``    Context / Factorization handles over the C ABI, and the
              LAPACK-shaped ``dgetrf``/``dgetrs`` wrappers.
``workloads`` seeded synthetic inputs of the benchmark configurations.
``build``     the nvcc build of libgblu.so (in-tree, no CMake).

The directory name is not a Python identifier; load it as a package with
``__graft_entry__.load_package()`` (it registers it as ``linearsolve_gb300``).
"""
from ._lib import GBLUError, load as load_library  # noqa: F401
from .device import Batch, Context, Factorization, default_context, dgetrf, dgetrs  # noqa: F401
from .linear import (  # noqa: F401
    DefaultAlgorithmChoice, DefaultLinearSolver, GB300LUFactorization, GB300MixedLUFactorization,
    GB300RFLUFactorization, LinearAliasSpecifier, RFLUCacheval, LinearCache, LinearProblem, LinearSolution, OperatorAssumptions,
    OperatorCondition, ReturnCode, defaultalg, init, reinit, solve, solve_bang, successful_retcode,
)
from ._cuda import DeviceMatrix, Event, PinnedArray  # noqa: F401
from . import workloads  # noqa: F401
