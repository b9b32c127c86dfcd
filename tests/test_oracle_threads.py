"""The oracle's per-particle loops on several threads give the same bits as
the serial restatement (CPU only): the large GPU parity cases run the
oracle on every host core."""
import numpy as np
import pytest

from meshlesshydro_gb300 import ic
from meshlesshydro_gb300.config import MFVConfig

ARRAYS = ("off", "nnl", "noi", "noi_img", "rev", "omega", "rho", "P", "dt", "B", "psi", "Aij", "WL", "WR",
          "vFrame", "F", "mF", "eF", "vF", "newton_iters", "stats", "grad_rho", "grad_P", "gradraw_vx")


def _run(oracle_mod, cfg, p, threads, steps):
    oracle_mod.set_threads(threads)
    try:
        o = oracle_mod.Oracle(cfg, p)
        for _ in range(steps):
            assert o.step() == 0
        out = {k: o.get(k) for k in ARRAYS}
        out.update(o.state())
        o.close()
        return out
    finally:
        oracle_mod.set_threads(1)


@pytest.mark.parametrize("case", ["kh24", "sedov12_nonperiodic", "sedov12_periodic_adaptive_h"])
def test_threads_bit_identical(oracle_mod, case):
    if case == "kh24":
        p = ic.kelvin_helmholtz(n_side=24, seed=3)
        cfg = MFVConfig.kelvin_helmholtz(p, pairwise_limiter=True)
    elif case == "sedov12_nonperiodic":
        p = ic.sedov(n_side=12, seed=4, energy=0.05)
        cfg = MFVConfig.sedov(p, periodic=False)
    else:
        p = ic.sedov(n_side=12, seed=4, energy=0.05)
        from dataclasses import replace
        cfg = replace(MFVConfig.sedov(p, periodic=True), adaptive_h=True, n_ngb=32.0,
                      kernel_size=p.kernel_size * 1.25)
    a = _run(oracle_mod, cfg, p, 1, 3)
    b = _run(oracle_mod, cfg, p, 4, 3)
    for k in a:
        assert np.array_equal(a[k], b[k], equal_nan=True), k
