"""The single-precision filters (mlh_tuning.fp32_filters).

On this GPU the FP64 pipe bounds the step and the FP32 pipe is 64 times
wider, so two reductions over neighbours are first bounded in single
precision and evaluated in FP64 only where the bound says the result can
come from:

* Particles::slopeLimiter (Particles.cpp:1313-1444) takes the largest and
  smallest face-point value f_ij = f_i + grad f . (x_ij - x_i) over the
  neighbours: f_ij in FP64 only at the neighbours where a bounded estimate
  can reach an extremum;
* Particles::compGlobalTimestep (Particles.cpp:1446-1485) takes the smallest
  dt_i = CFL h / max_j v_sig,ij over the particles: v_sig in FP64 only for
  the particles whose bounded dt can be the smallest.

The extrema, the time step and so every limited gradient and the whole
step are the same bits as with the filters off.  Covered: 2D and 3D,
periodic images and non-periodic boxes, the h/4 quadrature point,
per-particle smoothing lengths, fields with zero gradient (the Sedov
background's velocities and pressure in the first step), strong blasts,
and an ensemble (one time step per member).
"""
from dataclasses import replace

import numpy as np
import pytest

from meshlesshydro_gb300 import ic
from meshlesshydro_gb300.config import MFVConfig

pytestmark = pytest.mark.gpu

BASE = {"face_threads": 128, "face_blocks_per_sm": 4, "grad_threads": 64, "nns_warps_per_sm": 32,
        "face_split": 1, "link_overlap": 2}
FIELDS = {2: ("rho", "vx", "vy", "P"), 3: ("rho", "vx", "vy", "vz", "P")}


def _runtime():
    from meshlesshydro_gb300 import build, runtime
    build.build()
    return runtime


def _cases():
    kh = ic.kelvin_helmholtz(n_side=32, seed=3)
    sd = ic.sedov(n_side=20, seed=5)
    sd12 = ic.sedov(n_side=12, seed=4, energy=0.05)
    mb = ic.multi_blast(n_side=16, n_blasts=4, seed=11, energy=0.02)
    return {
        "kh32": (MFVConfig.kelvin_helmholtz(kh), kh, None),
        "kh32_pairwise_hq": (MFVConfig.kelvin_helmholtz(kh, pairwise_limiter=True, first_order_quad_point=False),
                             kh, None),
        "sedov20_periodic": (MFVConfig.sedov(sd, periodic=True), sd, None),
        "sedov20_nonperiodic": (MFVConfig.sedov(sd, periodic=False), sd, None),
        "sedov12_adaptive_h": (replace(MFVConfig.sedov(sd12, periodic=True), adaptive_h=True, n_ngb=32.0,
                                       kernel_size=sd12.kernel_size * 1.25), sd12, None),
        "multi_blast16": (MFVConfig.sedov(mb, periodic=True), mb, None),
        "kh_ensemble8": (None, None, ic.kh_ensemble(n_members=8, seed=3, n_min=400, n_max=2500)),
    }


@pytest.mark.parametrize("name", sorted(_cases()))
def test_fp32_filters_give_the_same_step(name):
    rt = _runtime()
    cfg, p, members = _cases()[name]
    runs = []
    for sf in (0, 3):
        if members is not None:
            s = rt.Simulation(MFVConfig.kelvin_helmholtz(members[0]), members=members)
        else:
            s = rt.Simulation(cfg, p)
        s.set_tuning(dict(BASE, fp32_filters=sf))
        grads = []
        for _ in range(4):
            st = s.step(1)
            assert st.steps == 1 and st.status == 0
            out = {f: s.get("grad_" + f) for f in FIELDS[cfg.dim if cfg else 2]}
            out["dt"] = s.get("dt")
            grads.append(out)
        runs.append((grads, s.get_state()))
        s.close()
    (ga, a), (gb, b) = runs
    for k, (x, y) in enumerate(zip(ga, gb)):
        for f in x:
            assert np.array_equal(x[f], y[f]), f"{name}: {f} differs at step {k + 1}"
    for k in a:
        assert np.array_equal(a[k], b[k]), f"{name}: state {k}"
