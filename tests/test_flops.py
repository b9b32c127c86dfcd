"""The operation-counting build of the oracle (oracle/flop_count.hpp,
oracle/flops.py): it computes the same step bit for bit, its counts agree
with hand counts of simple stages, and bench.py's algorithmic flops per face
are what it counts on the stated samples."""
import numpy as np
import pytest

from meshlesshydro_gb300 import ic
from meshlesshydro_gb300.config import MFVConfig


def _pair(oracle_mod, cfg, p, steps):
    plain = oracle_mod.Oracle(cfg, p)
    counted = oracle_mod.Oracle(cfg, p, counting=True)
    for _ in range(steps):
        assert plain.step() == counted.step()
    return plain, counted


@pytest.mark.parametrize("case", ["sedov12_periodic", "sedov10_nonperiodic", "kh24"])
def test_counting_build_is_bit_identical(oracle_mod, case):
    """Computing in the counting double changes no result: every array of the
    step (neighbour lists, gradients, face states, fluxes, the new state)."""
    if case == "sedov12_periodic":
        p = ic.sedov(n_side=12, seed=4, energy=0.05)
        cfg = MFVConfig.sedov(p, periodic=True)
    elif case == "sedov10_nonperiodic":
        p = ic.sedov(n_side=10, seed=6)
        cfg = MFVConfig.sedov(p, periodic=False)
    else:
        p = ic.kelvin_helmholtz(n_side=24, seed=3)
        cfg = MFVConfig.kelvin_helmholtz(p)
    a, b = _pair(oracle_mod, cfg, p, 3)
    names = ["x", "y", "vx", "vy", "m", "u", "rho", "P", "omega", "nnl", "off", "noi", "noi_img", "B", "psi",
             "Aij", "WL", "WR", "vFrame", "F", "mF", "eF", "vF", "dt", "newton_iters", "stats",
             "grad_rho", "grad_P", "gradraw_vx"]
    if cfg.dim == 3:
        names += ["z", "vz"]
    for k in names:
        np.testing.assert_array_equal(a.get(k), b.get(k), err_msg=k)
    with pytest.raises(RuntimeError):
        a.flop_counts()   # the plain build has no counts


def test_counts_of_simple_stages(oracle_mod):
    """Hand counts: compPressure is (gamma - 1) rho u, two multiplications per
    particle (gamma - 1 is a constant); the 3D update is 38 operations per
    particle while no particle crosses the periodic boundary (kinetic energy
    8, momenta 3, mass 2, momentum kick 6, velocities 3, energy kick 2,
    internal energy 8, drift 6)."""
    import flops
    p = ic.sedov(n_side=12, seed=4, energy=0.05)
    cfg = MFVConfig.sedov(p, periodic=True)
    res = flops.count(cfg, p, 2)
    assert res["stages_per_particle"]["pressure"] == 2.0
    assert res["stages_per_particle"]["update"] == 38.0
    ops = res["ops_per_unit"]["faces_riemann"]
    assert ops["pow"] > 0 and ops["sqrt"] > 0 and ops["div"] > 0


@pytest.mark.parametrize("dim", [3, 2])
def test_bench_reference_ops_are_the_counted_ones(oracle_mod, dim):
    """bench.py's KERNEL_REF_OPS (the reference method's operations per unit,
    reported beside the rooflines): 16 steps of the 32^3 periodic Sedov
    lattice (3D) and of the 100x100 Kelvin-Helmholtz set-up (2D)."""
    import bench
    import flops
    if dim == 3:
        cfg, p = flops.workload("sedov", 32, 2)
    else:
        cfg, p = flops.workload("kh", 100, 1)
    res = flops.count(cfg, p, 16)
    for k, v in bench.KERNEL_REF_OPS[dim].items():
        got = res["per_unit"][k] if k in res["per_unit"] else 0.0
        assert abs(v - got) <= 0.002 * max(got, 1.0), (k, v, got)


def test_kernel_rooflines_arithmetic():
    """bench.kernel_rooflines: rates and fractions from the per-step times on
    the executed FP64 operations, kernels without a time left out."""
    import bench
    kt = {"neighbours_density": 2.0, "faces_riemann": 10.0, "face_links": 0.0, "grid_bin": 0.3}
    r = bench.kernel_rooflines(kt, 3, 1.0e6, 2.0e7, 1.0, 5000.0)
    assert set(r) == {"neighbours_density", "faces_riemann"}
    f = r["faces_riemann"]
    fl, by = bench.KERNEL_EXEC[3]["faces_riemann"]
    assert f["unit"] == "face" and f["units_per_step"] == 2.0e7
    assert abs(f["fp64_tflops"] - fl * 2.0e7 / 10.0e-3 / 1e12) < 1e-12
    assert abs(f["fp64_frac"] - f["fp64_tflops"]) < 1e-12
    assert abs(f["hbm_gbs"] - by * 2.0e7 / 10.0e-3 / 1e9) < 1e-9
    assert abs(f["hbm_frac"] - f["hbm_gbs"] / 5000.0) < 1e-12
    assert bench.kernel_rooflines(kt, 3, 1.0e6, 2.0e7, None, None)["faces_riemann"]["fp64_frac"] is None


def test_executed_rates_stay_below_the_fp64_peak():
    """The roofline unit passes the step-level check: on a measured Sedov
    128^3 step (2,097,152 particles, 33,556,373 faces, 41.74 ms; kernel times
    per step: face passes 24.0, gradients with the time step 10.6, neighbours
    4.4, gather and update 0.83 ms; FP64 FMA probe 1.058 TFLOP/s), every kernel's
    executed FP64 rate and the whole step's (the executed operations of all
    kernels over ms_per_step) stay at or below the peak.  The reference
    method's operation count would not (kept for comparison only)."""
    import bench
    n, faces, peak = 2097152.0, 33556373.0, 1.058
    kt = {"faces_riemann": 24.0, "gradients_limiter": 10.6, "neighbours_density": 4.4,
          "gather_update": 0.83}
    r = bench.kernel_rooflines(kt, 3, n, faces, peak, 6788.3)
    for k, v in r.items():
        assert v["fp64_frac"] <= 1.0, (k, v["fp64_frac"])
    step = bench.step_fp64(3, n, faces) / 41.74e-3 / 1e12
    assert step <= peak, step
    ref = sum(bench.KERNEL_REF_OPS[3][k] * (faces if u == "face" else n)
              for k, u in bench.KERNEL_UNITS.items()) / 41.74e-3 / 1e12
    assert ref > peak   # why the reference's count is no roofline
