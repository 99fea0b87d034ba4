"""Generate tests/golden/lu_golden.npz.

LinearSolve.jl's LUFactorization factors through LinearAlgebra.lu! ->
LAPACK.getrf! (src/factorization.jl:632-636,748) and solves through getrs
(:603-611); Julia is not available here, so the fixtures are produced by the
same LAPACK routines (scipy.linalg.lapack dgetrf/dgetrs on OpenBLAS) on
seeded inputs, plus the known answers of the reference's own tests:

  test/Core/resolve.jl:78-106      A = [1 2; 3 4]; A'A x = [1, 2]  =>  x = [-2, 1.5]
  test/Core/lu_refactorization.jl  Asing[:, 1] .= 0  =>  singular (info = 1, Failure)

Run:  python tests/golden/make_golden.py
"""
import os

import numpy as np
from scipy.linalg import lapack

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    rng = np.random.default_rng(20260101)
    out = {}
    cases = []
    # square sizes from test/Core/blocked_lufact.jl:44-54 (subset) + rectangular :119-130
    shapes = [(n, n) for n in (1, 2, 3, 5, 7, 8, 9, 13, 16, 17, 31, 32, 33, 40, 63, 64, 65, 100, 129)]
    shapes += [(100, 3), (3, 100), (128, 40), (40, 128), (65, 64), (64, 65)]
    for idx, (m, n) in enumerate(shapes):
        A = rng.standard_normal((m, n))
        lu, piv, info = lapack.dgetrf(A)
        key = f"c{idx}"
        out[key + "_A"] = A
        out[key + "_LU"] = lu
        out[key + "_ipiv"] = piv.astype(np.int64) + 1
        out[key + "_info"] = np.int64(info)
        if m == n:
            b = rng.standard_normal((n, 2))
            x, _ = lapack.dgetrs(lu, piv, b)
            xt, _ = lapack.dgetrs(lu, piv, b, trans=1)
            out[key + "_b"] = b
            out[key + "_x"] = x
            out[key + "_xt"] = xt
        cases.append(key)
    # known answer of test/Core/resolve.jl:78-106
    A = np.array([[1.0, 2.0], [3.0, 4.0]])
    out["known_A"] = A.T @ A
    out["known_b"] = np.array([1.0, 2.0])
    out["known_x"] = np.array([-2.0, 1.5])
    # singular case of test/Core/lu_refactorization.jl:83-110 (n = 8, A = rand + n I, column 1 zeroed)
    Ag = rng.random((8, 8)) + 8 * np.eye(8)
    As = Ag.copy()
    As[:, 0] = 0.0
    lu, piv, info = lapack.dgetrf(As)
    out["sing_Agood"] = Ag
    out["sing_A"] = As
    out["sing_info"] = np.int64(info)
    out["cases"] = np.array(cases)
    np.savez_compressed(os.path.join(HERE, "lu_golden.npz"), **out)
    print("wrote", len(cases), "cases; singular info =", info)


if __name__ == "__main__":
    main()
