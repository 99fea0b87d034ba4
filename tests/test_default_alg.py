"""The default algorithm choice (src/default.jl:277-284, :411-520) restated
for the GB300 algorithms; host logic only."""
import numpy as np
import pytest


def test_defaultalg_choices(pkg):
    A = np.zeros((5, 5))
    b = np.zeros(5)
    d = pkg.defaultalg(A, b)
    assert d.alg == pkg.DefaultAlgorithmChoice.GB300LUFactorization
    assert isinstance(d.concrete(), pkg.GB300LUFactorization)
    well = pkg.OperatorAssumptions(True, pkg.OperatorCondition.WellConditioned)
    d = pkg.defaultalg(A, b, well)
    assert d.alg == pkg.DefaultAlgorithmChoice.GB300MixedLUFactorization
    m = d.concrete()
    assert isinstance(m, pkg.GB300MixedLUFactorization) and m.fallback
    for cond in (pkg.OperatorCondition.VeryIllConditioned, pkg.OperatorCondition.SuperIllConditioned):
        with pytest.raises(NotImplementedError):
            pkg.defaultalg(A, b, pkg.OperatorAssumptions(True, cond))
    with pytest.raises(NotImplementedError):
        pkg.defaultalg(np.zeros((6, 5)), np.zeros(6))
