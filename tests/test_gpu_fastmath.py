"""The kernels' reciprocal, quotient and reciprocal square root (one third-order step
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


def test_power_of_two_scalings_are_ieee_products():
    """scale_down<1>, scale_down<2> and twice (integer-pipe stand-ins for a
    DMUL by 0.5, 0.25 and 2) give the IEEE products bit for bit, subnormal
    results (rounded to nearest even) and overflow included."""
    from meshlesshydro_gb300 import build, runtime
    build.build()
    L = runtime.load()
    rng = np.random.default_rng(5)
    tiny = np.arange(0, 4096, dtype=np.uint64)                       # subnormals, both ends of the binade
    edge = np.concatenate([tiny, tiny + np.uint64(0x000FFFFFFFFFF000), tiny + np.uint64(0x0010000000000000),
                           tiny + np.uint64(0x001FFFFFFFFFF000), tiny + np.uint64(0x0020000000000000),
                           tiny + np.uint64(0x7FEFFFFFFFFFF000)]).view(np.float64)
    special = np.array([0.0, np.inf, 1.0, 2.0 ** -1022, 2.0 ** -1021, 2.0 ** 1023, np.finfo(np.float64).max])
    randn = rng.standard_normal(20000) * 10.0 ** rng.uniform(-300, 300, 20000)
    x = np.concatenate([edge, special, randn])
    x = np.concatenate([x, -x])
    n = x.size
    h, q, t = np.empty(n), np.empty(n), np.empty(n)
    dp = lambda a: a.ctypes.data
    assert L.mlh_probe_scale2(n, dp(x), dp(h), dp(q), dp(t)) == 0
    with np.errstate(over="ignore"):
        for got, want in ((h, x * 0.5), (q, x * 0.25), (t, x * 2.0)):
            np.testing.assert_array_equal(got.view(np.uint64), want.view(np.uint64))
    nan = np.array([np.nan, -np.nan])
    h2, q2, t2 = np.empty(2), np.empty(2), np.empty(2)
    assert L.mlh_probe_scale2(2, dp(nan), dp(h2), dp(q2), dp(t2)) == 0
    assert np.isnan(h2).all() and np.isnan(q2).all() and np.isnan(t2).all()
