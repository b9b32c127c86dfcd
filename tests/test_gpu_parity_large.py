"""GPU parity at the sizes of the measured workloads: the CUDA MFV step
(libmlh.so, through the C ABI) against the CPU oracle on identical seeded
inputs.

* Sedov 64^3 (262,144 particles), periodic and in the reference's own
  non-periodic mode (testcases/sedov/parameter.h:12): one step stage by stage,
  then up to 100 steps in which the GPU starts every step from the oracle's
  state (the per-step gate of tests/helpers.py, neighbour lists bit-exact
  every step), and a free-running run over the same steps whose density is
  compared by L1 (<= 1e-8 relative).  The reference's scheme gives negative
  internal energy at the blast's evacuated centre at its 65th step (index
  64), which ends the comparison.
* Sedov 128^3 (2,097,152 particles, the bench workload): one step, lists
  bit-exact, fields per element.
* Kelvin-Helmholtz 100x100: 100 steps per-step gated, and every state field
  of a free-running 100-step run by L1.
* The meshless finite mass scheme (MESHLESS_FINITE_MASS 1) and fixed
  particles (MOVE_PARTICLES 0) over five whole steps.

The oracle runs its per-particle loops on every host core (its results do not
depend on the thread count: tests/test_oracle_threads.py).
"""
import numpy as np
import pytest

from meshlesshydro_gb300 import ic
from meshlesshydro_gb300.config import MFVConfig
from helpers import (MAX_TIE_FRACTION, assert_close, assert_state, compare_step, flux_terms, l1_rel, pset_from_state,
                     rank_deficient, state_of, state_terms, step_limits)

pytestmark = pytest.mark.gpu

L1_RTOL = 1e-8


@pytest.fixture(scope="module")
def orc(oracle_mod):
    oracle_mod.set_threads(0)
    yield oracle_mod
    oracle_mod.set_threads(1)


def _sim(cfg, p):
    from meshlesshydro_gb300 import build, runtime
    build.build()
    return runtime.Simulation(cfg, p)


def _sedov64(periodic):
    p = ic.sedov(n_side=64, seed=2)
    return p, MFVConfig.sedov(p, periodic=periodic)


@pytest.mark.parametrize("periodic", [True, False], ids=["periodic", "nonperiodic"])
def test_sedov64_one_step_stagewise(orc, periodic):
    p, cfg = _sedov64(periodic)
    o = orc.Oracle(cfg, p)
    assert o.step() == 0
    g = _sim(cfg, p)
    st = g.step(1)
    compare_step(g, o, 3, slots=True, what=f"sedov64 periodic={periodic}: ", pre=state_of(p))
    assert st.faces == int(o.get("stats")[0])
    g.close()
    o.close()


def _per_step_and_free_run(orc, p, cfg, nsteps, what, free_fields=("rho",)):
    """nsteps oracle steps; before each, the GPU takes the oracle's state and
    runs one step, gated per element (lists bit-exact).  A step at which the
    reference's own scheme gives non-physical values (the oracle's status) is
    gated too and ends the comparison.
    Then a free-running GPU run over the steps before it, from the initial
    state, compared with the oracle's states by L1.  Returns the L1 errors
    and the number of steps compared."""
    o = orc.Oracle(cfg, p)
    g = _sim(cfg, p)
    ties = 0
    done = nsteps
    ost = orho = None
    for k in range(nsteps):
        pre = o.state()
        g.set_state(pset_from_state(p, pre))
        so = o.step()
        sg = g.step(1, check=False).status
        assert so != 0 or sg == 0, f"{what}: GPU status {sg:#x} at step {k}"
        np.testing.assert_array_equal(g.get("nnl"), o.get("nnl"), err_msg=f"{what}: nnl at step {k}")
        assert_close(g.get("rho"), o.get("rho"), floor=0.0, what=f"{what} step {k}: rho")
        assert_close(g.get("dt"), o.get("dt"), floor=0.0, what=f"{what} step {k}: dt")
        lim, _, tie = step_limits(g, o, cfg.dim)
        ties += int(tie.sum() // 2)
        nrd = int(rank_deficient(o, cfg.dim).sum())
        assert nrd <= 1e-4 * p.n, f"{what}: {nrd} particles with fewer than {cfg.dim} neighbours at step {k}"
        ost_k = o.state()
        terms = state_terms(pre, ost_k, flux_terms(o.get("F"), o.get("off"), cfg.dim), float(o.get("dt")[0]),
                            cfg.dim)
        assert_state(g.get_state(), ost_k, lim, what=f"{what} step {k}: ", terms=terms)
        if so != 0:
            # the reference's scheme gives non-physical values at this step
            # (its cause, a particle with a singular E_i, is out of the gate
            # above and its outcome is rounding noise in both codes, so the
            # GPU's status is not required to match): no step after it is
            # compared
            done, ost, orho = k, pre, o.get("rho")
            break
    faces = max(int(o.get("stats")[0]), 1)
    assert ties <= MAX_TIE_FRACTION * faces * max(done, 1) + 1, f"{what}: {ties} Newton ties in {done} steps"
    if ost is None:
        # the oracle's state after nsteps, and its density at the next step's
        # density evaluation
        ost = o.state()
        o.step()
        orho = o.get("rho")
    # the free run: the GPU the same from the initial state
    g.set_state(p)
    if done:
        g.step(done)
    gst = g.get_state()
    g.step(1, check=False)
    grho = g.get("rho")
    out = {"rho": l1_rel(grho, orho)}
    for f in free_fields:
        if f != "rho":
            out[f] = l1_rel(gst[f], ost[f])
    g.close()
    o.close()
    return out, done


@pytest.mark.parametrize("periodic", [True, False], ids=["periodic", "nonperiodic"])
def test_sedov64_100_steps(orc, periodic):
    """100 steps, or up to the step at which the reference's scheme itself
    gives non-physical values.  The particle at the blast's evacuated centre
    keeps 3 neighbours up to step index 63 (cond(E_i) = 1.2e8, gated with
    the condition-number tolerance) and has one at index 64, where E_i is
    singular, the reference inverts rounding noise and the oracle reports
    negative internal energy (and, non-periodic, negative mass).  That step
    is gated with the particle and its neighbour out of the gate
    (tests/helpers.py), the GPU need not report the same status, and the
    comparison ends there.  The free run compares the steps before it."""
    p, cfg = _sedov64(periodic)
    l1, done = _per_step_and_free_run(orc, p, cfg, 100, f"sedov64 periodic={periodic}")
    print(f"sedov64 periodic={periodic}: {done} steps compared, density L1 {l1['rho']:.3e}")
    assert done >= 60
    assert l1["rho"] <= L1_RTOL, f"density L1 after {done} steps {l1['rho']:.3e}"


def test_sedov128_one_step(orc):
    p = ic.sedov(n_side=128, seed=2)
    cfg = MFVConfig.sedov(p, periodic=True)
    o = orc.Oracle(cfg, p)
    assert o.step() == 0
    g = _sim(cfg, p)
    st = g.step(1)
    compare_step(g, o, 3, slots=False, what="sedov128: ", pre=state_of(p))
    assert st.faces == int(o.get("stats")[0])
    g.close()
    o.close()


def test_kh100_100_steps_all_fields(orc):
    p = ic.kelvin_helmholtz(n_side=100, seed=1)
    cfg = MFVConfig.kelvin_helmholtz(p)
    l1, done = _per_step_and_free_run(orc, p, cfg, 100, "kh100", free_fields=("rho", "x", "y", "vx", "vy", "m", "u"))
    assert done == 100
    for f, e in l1.items():
        assert e <= L1_RTOL, f"{f}: L1 after 100 steps {e:.3e}"


@pytest.mark.parametrize("mode", ["meshless_finite_mass", "fixed_particles"])
def test_kh24_mfm_and_fixed_particles(orc, mode):
    """MESHLESS_FINITE_MASS 1 (Particles.cpp:2041-2043, Riemann.cpp:171-175:
    no mass flux, masses kept) and MOVE_PARTICLES 0 (Particles.cpp:1542-1565,
    2077-2108: frame velocity 0, no drift), five whole steps: the first stage
    by stage, every step per element from the oracle's state, then a free run."""
    p = ic.kelvin_helmholtz(n_side=24, seed=3)
    kw = {"meshless_finite_mass": True} if mode == "meshless_finite_mass" else {"move_particles": False}
    cfg = MFVConfig.kelvin_helmholtz(p, **kw)
    o = orc.Oracle(cfg, p)
    assert o.step() == 0
    g = _sim(cfg, p)
    g.step(1)
    compare_step(g, o, 2, slots=True, what=mode + ": ", pre=state_of(p))
    gs = g.get_state()
    if mode == "meshless_finite_mass":
        assert np.array_equal(gs["m"], p.m)
    else:
        assert np.array_equal(gs["x"], p.x) and np.array_equal(gs["y"], p.y)
    g.close()
    o.close()
    l1, done = _per_step_and_free_run(orc, p, cfg, 5, mode, free_fields=("rho", "x", "y", "vx", "vy", "m", "u"))
    assert done == 5
    for f, e in l1.items():
        assert e <= L1_RTOL, f"{mode} {f}: L1 after 5 steps {e:.3e}"
