"""The `mlh` command-line driver (config.info + parameter.h + HDF5 in and out,
the time loop of MeshlessScheme::run) on the GPU, against the oracle."""
import os
import subprocess

import numpy as np
import pytest

import h5spec
from meshlesshydro_gb300 import build, ic, io
from meshlesshydro_gb300.config import MFVConfig
from helpers import assert_close, assert_normwise

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

KH_PARAMS = """#define DIM 2
#define PERIODIC_BOUNDARIES 1
#define SLOPE_LIMITING 1
#define BETA 4.
#define ENFORCE_FLUX_SYM 1
#define MOVE_PARTICLES 1
#define FIRST_ORDER_QUAD_POINT 1
#define MAX_NUM_INTERACTIONS 60
"""

SEDOV_PARAMS = """#define DIM 3
#define PERIODIC_BOUNDARIES 0
#define ADAPTIVE_TIMESTEP 1
#define CFL .25
#define SLOPE_LIMITING 1
#define BETA 1.
#define PAIRWISE_LIMITER 1
#define PSI_1 .5
#define PSI_2 .25
#define MOVE_PARTICLES 1
#define FIRST_ORDER_QUAD_POINT 1
"""


def run_driver(tmp_path, pset, params, time_step, time_end, interval):
    build.build()
    icf = tmp_path / "ic.h5"
    io.write_initial_distribution(str(icf), pset)
    box = "".join(f"    lower{a} {pset.box_lo[k]!r}\n    upper{a} {pset.box_hi[k]!r}\n" for k, a in enumerate("XYZ"))
    (tmp_path / "config.info").write_text(
        f"initFile {icf}\noutDir {tmp_path / 'out'}\ntimeStep {time_step!r}\ntimeEnd {time_end!r}\n"
        f"h5DumpInterval {interval}\nperiodicBoxLimits {{\n{box}}}\nkernelSize {pset.kernel_size!r}\n"
        f"gamma {pset.gamma!r}\n")
    (tmp_path / "parameter.h").write_text(params)
    exe = os.path.join(ROOT, "meshlesshydro_gb300", "mlh")
    r = subprocess.run([exe, "-c", str(tmp_path / "config.info"), "-p", str(tmp_path / "parameter.h")],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out = tmp_path / "out"
    return {f: h5spec.read(str(out / f)) for f in sorted(os.listdir(out))}


def test_driver_fixed_dt_matches_oracle(tmp_path, oracle_mod):
    """KH with a fixed timeStep: a dump every 5 steps (step % h5DumpInterval
    == 0) of the state and the density of that step, 10 steps, against the
    oracle stepping the same 10 steps."""
    p = ic.kelvin_helmholtz(n_side=24, seed=3)
    snaps = run_driver(tmp_path, p, KH_PARAMS, 0.002, 0.02, 5)
    assert list(snaps) == ["000000.h5", "000005.h5", "000010.h5"]
    cfg = MFVConfig.kelvin_helmholtz(p, adaptive_timestep=False, time_step=0.002)
    o = oracle_mod.Oracle(cfg, p)
    for k in range(10):
        assert o.step() == 0
        if k == 0:
            s0 = snaps["000000.h5"]
            assert s0["time"][0] == 0.0
            assert_close(s0["rho"], o.get("rho"), what="rho at t = 0")
            assert_close(s0["rhoGrad"], o.get("grad_rho").reshape(-1, 3)[:, :2], what="rhoGrad at t = 0")
            np.testing.assert_array_equal(s0["noi"], o.get("noi"))
    last = snaps["000010.h5"]
    st = o.state()
    # the state after 10 steps (differences compound over steps)
    assert_normwise(last["x"][:, 0], st["x"], 1e-12, what="x")
    assert_normwise(last["v"][:, 1], st["vy"], 1e-12, what="vy")
    assert_normwise(last["m"], st["m"], 1e-12, what="m")
    assert_normwise(last["u"], st["u"], 1e-12, what="u")
    assert abs(last["totalMass"][0] - np.sum(p.m)) <= 1e-13 * np.sum(p.m)


def test_driver_adaptive_dump_schedule(tmp_path):
    """Sedov (non-periodic, adaptive dt): dumps land on the dump times of
    MeshlessScheme::run, k * timeStep * h5DumpInterval, the steps are
    clamped to them, mass and energy are conserved to rounding."""
    p = ic.sedov(n_side=10, seed=4, energy=0.05)
    snaps = run_driver(tmp_path, p, SEDOV_PARAMS, 0.001, 0.004, 1)
    times = [s["time"][0] for s in snaps.values()]
    assert len(times) >= 3 and times[0] == 0.0
    dump_times = [k * 0.001 for k in range(5)]
    for t in times[1:]:
        assert min(abs(t - d) for d in dump_times) <= 1e-15
    e = [s["energy"][0] for s in snaps.values()]
    m = [s["totalMass"][0] for s in snaps.values()]
    assert max(abs(x - m[0]) for x in m) <= 1e-13 * m[0]
    assert max(abs(x - e[0]) for x in e) <= 1e-12 * e[0]
    # the last snapshot reads back as an initial distribution
    last = os.path.join(tmp_path, "out", list(snaps)[-1])
    st, mat = io.read_initial_distribution(last, 3)
    assert st["x"].shape == (p.n,) and np.all(mat == 0)
