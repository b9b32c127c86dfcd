"""The kernels' reciprocal, quotient and reciprocal square root (Newton-Raphson
from the hardware estimates, mlh_device.cuh frcp / fdiv / frsqrt) against
exact values: the error bound is 2 ulp (reciprocal, reciprocal square root)
and 3 ulp (quotient), over the decades the MFV step meets."""
import ctypes
from decimal import Decimal, getcontext

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def ulp_error(got, exact):
    return np.abs(got - exact) / np.spacing(np.abs(exact))


def test_fast_math_error_bounds():
    from meshlesshydro_gb300 import build, runtime
    build.build()
    L = runtime.load()
    rng = np.random.default_rng(17)
    n = 4000
    x = 10.0 ** rng.uniform(-30, 30, n)
    x[:64] = 2.0 ** np.arange(-32, 32)                  # powers of two
    x[64:128] = np.nextafter(2.0 ** np.arange(-32, 32), 0)   # just below them
    y = rng.normal(0.0, 1.0, n) * 10.0 ** rng.uniform(-10, 10, n)
    rcp, quot, rsq = np.empty(n), np.empty(n), np.empty(n)
    dp = lambda a: a.ctypes.data
    assert L.mlh_probe_fast_math(n, dp(x), dp(y), dp(rcp), dp(quot), dp(rsq)) == 0
    getcontext().prec = 40
    ex_rcp = np.array([float(Decimal(1) / Decimal(v)) for v in x])
    ex_quot = np.array([float(Decimal(b) / Decimal(a)) for a, b in zip(x, y)])
    ex_rsq = np.array([float(Decimal(1) / Decimal(v).sqrt()) for v in x])
    assert np.max(ulp_error(rcp, ex_rcp)) <= 2
    assert np.max(ulp_error(quot, ex_quot)) <= 3
    assert np.max(ulp_error(rsq, ex_rsq)) <= 2
    # most results are the correctly rounded ones
    assert np.mean(rcp == ex_rcp) > 0.8
