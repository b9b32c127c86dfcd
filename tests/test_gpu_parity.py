"""GPU parity: the CUDA MFV step (libmlh.so, through the C ABI) against the
CPU oracle on identical seeded inputs.

Bar: neighbour lists bit-exact (indices, order, image flags); every per-step
field within the per-element gate of helpers.assert_close (1e-12 of each
entry, with a floor of 1e-3 of the field's largest magnitude).
The oracle itself is pinned to the reference's own code by
tests/test_oracle_golden.py.
"""
import numpy as np
import pytest

from meshlesshydro_gb300 import ic
from meshlesshydro_gb300.config import MFVConfig
from helpers import assert_normwise, compare_step, state_of

pytestmark = pytest.mark.gpu


def _sim(cfg, p):
    from meshlesshydro_gb300 import build, runtime
    build.build()
    return runtime.Simulation(cfg, p)


def cases():
    kh24 = ic.kelvin_helmholtz(n_side=24, seed=3)
    kh100 = ic.kelvin_helmholtz(n_side=100, seed=1)
    sd12 = ic.sedov(n_side=12, seed=4, energy=0.05)
    sd16 = ic.sedov(n_side=16, seed=5)
    # gamma = 1.4: the general-gamma Riemann path (pow instead of fifth roots)
    kh24g = ic.kelvin_helmholtz(n_side=24, seed=3, gamma=1.4)
    sd12g = ic.sedov(n_side=12, seed=4, energy=0.05, gamma=1.4)
    return {
        "kh24": (kh24, MFVConfig.kelvin_helmholtz(kh24)),
        "kh24_int_abs": (kh24, MFVConfig.kelvin_helmholtz(kh24, int_abs=True)),
        "kh24_pairwise": (kh24, MFVConfig.kelvin_helmholtz(kh24, pairwise_limiter=True)),
        # the face point x_i + kernelSize/4 (x_j - x_i) (FIRST_ORDER_QUAD_POINT 0)
        "kh24_pairwise_q": (kh24, MFVConfig.kelvin_helmholtz(kh24, pairwise_limiter=True,
                                                             first_order_quad_point=False)),
        "kh24_gamma14": (kh24g, MFVConfig.kelvin_helmholtz(kh24g)),
        # SLOPE_LIMITING 0 (MeshlessScheme.cpp:124-130, 140-144 skip slopeLimiter)
        "kh24_no_slope_limiter": (kh24, MFVConfig.kelvin_helmholtz(kh24, slope_limiting=False)),
        # ADAPTIVE_TIMESTEP 0: the configured timeStep (MeshlessScheme.cpp:91-105)
        "kh24_fixed_dt": (kh24, MFVConfig.kelvin_helmholtz(kh24, adaptive_timestep=False, time_step=1e-3)),
        "kh100": (kh100, MFVConfig.kelvin_helmholtz(kh100)),
        "sedov12_nonperiodic_nopw": (sd12, MFVConfig.sedov(sd12, periodic=False, pairwise_limiter=False)),
        "sedov12_gamma14_nonperiodic": (sd12g, MFVConfig.sedov(sd12g, periodic=False)),
        "sedov16_nonperiodic": (sd16, MFVConfig.sedov(sd16, periodic=False)),
        "sedov16_periodic": (sd16, MFVConfig.sedov(sd16, periodic=True)),
        "sedov16_periodic_int_abs": (sd16, MFVConfig.sedov(sd16, periodic=True, int_abs=True)),
    }


CASES = cases()


@pytest.mark.parametrize("name", sorted(CASES))
def test_one_step_stagewise(oracle_mod, name):
    p, cfg = CASES[name]
    o = oracle_mod.Oracle(cfg, p)
    assert o.step() == 0
    g = _sim(cfg, p)
    stats = g.step(1)
    assert stats.steps == 1
    compare_step(g, o, cfg.dim, slots=True, what=name + ": ", pre=state_of(p))
    assert stats.faces == int(o.get("stats")[0])


def test_flux_antisymmetry_bitwise():
    """Particles::checkFluxSymmetry (Particles.cpp:2888-2976): F_ji = -F_ij exactly."""
    p, cfg = CASES["sedov16_periodic"]
    g = _sim(cfg, p)
    g.step(1)
    off = g.get("off")
    nnl = g.get("nnl")
    noi = g.get("noi")
    F = g.get("F").reshape(-1, cfg.dim + 2)
    idx = nnl & ((1 << 29) - 1)
    n = p.n
    checked = 0
    for i in range(0, n, 7):
        for s in range(off[i], off[i + 1]):
            j = int(idx[s])
            img = (s - off[i]) >= noi[i]
            lo, hi = (off[j] + noi[j], off[j + 1]) if img else (off[j], off[j] + noi[j])
            t = lo + int(np.nonzero(idx[lo:hi] == i)[0][0])
            assert np.array_equal(F[s], -F[t])
            checked += 1
    assert checked > 1000


def _totals(st, dim):
    m = st["m"]
    v = [st["vx"], st["vy"]] + ([st["vz"]] if dim == 3 else [])
    E = m * (st["u"] + 0.5 * sum(c * c for c in v))
    import math
    return {"mass": math.fsum(m), "energy": math.fsum(E),
            **{f"p{a}": math.fsum(m * c) for a, c in zip("xyz", v)},
            **{f"s{a}": math.fsum(np.abs(m * c)) for a, c in zip("xyz", v)}}


@pytest.mark.parametrize("name", ["kh100", "sedov16_periodic"])
def test_conservation(name):
    """Mass and energy to 1e-13 relative per step; each momentum component
    to 1e-13 of sum |m v_a| (the total itself is near zero: a symmetric blast,
    counter-flowing KH layers), plus 1e-18 for a state at rest."""
    p, cfg = CASES[name]
    g = _sim(cfg, p)
    t0 = _totals(g.get_state(), cfg.dim)
    for _ in range(10):
        g.step(1)
        t1 = _totals(g.get_state(), cfg.dim)
        assert abs(t1["mass"] - t0["mass"]) <= 1e-13 * abs(t0["mass"])
        assert abs(t1["energy"] - t0["energy"]) <= 1e-13 * abs(t0["energy"])
        for a in "xyz"[:cfg.dim]:
            assert abs(t1["p" + a] - t0["p" + a]) <= 1e-13 * t0["s" + a] + 1e-18, a
        t0 = t1


def test_deterministic_bitwise():
    p, cfg = CASES["sedov16_periodic"]
    a = _sim(cfg, p)
    b = _sim(cfg, p)
    a.step(3)
    b.step(3)
    sa, sb = a.get_state(), b.get_state()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k


@pytest.mark.parametrize("name", ["sedov16_periodic", "kh100"])
def test_face_pass_structures_bitwise(name):
    """The three structures of the plain face pass (one pass; a second
    Newton pass over a queue; the unfinished faces continued inside the
    block) run the same arithmetic on every face: identical states, bit for
    bit, over steps where both converged and unfinished faces occur."""
    p, cfg = CASES[name]
    states, iters = [], []
    for split in (0, 1, 2):
        sim = _sim(cfg, p)
        sim.set_tuning({"face_threads": 128, "face_blocks_per_sm": 4, "grad_threads": 64,
                        "nns_warps_per_sm": 32, "face_split": split})
        st = sim.step(3)
        states.append(sim.get_state())
        iters.append(st.newton_iterations)
        sim.close()
    for other in states[1:]:
        for k in states[0]:
            assert np.array_equal(states[0][k], other[k]), k
    assert iters[0] == iters[1] == iters[2]


def test_neighbour_overflow_retry(oracle_mod):
    """Too few slots: the step detects the overflow, grows the slots and
    repeats (the reference exits, Particles.cpp:348-352)."""
    p, cfg = CASES["kh24"]
    from dataclasses import replace
    g = _sim(replace(cfg, max_neighbours=6), p)
    g.step(2)
    o = oracle_mod.Oracle(cfg, p)
    o.step(); o.step()
    np.testing.assert_array_equal(g.get("nnl"), o.get("nnl"))
    gs = g.get_state()
    for k, v in o.state().items():
        assert_normwise(gs[k], v, 1e-11, what=k)


def test_negative_pressure_reported():
    """A negative internal energy gives P < 0: the status word reports it
    (the reference only warns, Particles.cpp:1284-1286)."""
    p, cfg = CASES["kh24"]
    q = p.copy()
    q.u[5] = -1.0
    from meshlesshydro_gb300 import runtime
    g = _sim(cfg, q)
    st = g.step(1, check=False)
    assert st.status & (1 << 1)


def test_nan_reported():
    """A NaN in the state (an internal energy here) reaches the updated
    state, and the update reports it in the status word; every loop of the
    step is bounded, so the step still ends (the reference has no check)."""
    p, cfg = CASES["kh24"]
    q = p.copy()
    q.u[5] = np.nan
    g = _sim(cfg, q)
    st = g.step(1, check=False)
    assert st.status & (1 << 10)


@pytest.mark.parametrize("name,nsteps,rtol", [("kh100", 100, 1e-8), ("kh24_gamma14", 50, 1e-8),
                                              ("sedov16_periodic", 30, 1e-8),
                                              ("sedov16_nonperiodic", 40, 1e-8)])
def test_multistep_density_l1(oracle_mod, name, nsteps, rtol):
    """Density after many steps: L1 relative difference to the oracle.  The
    non-periodic 16^3 blast becomes unstable at the edge of the particle
    cloud after about 61-63 steps in the oracle and on the GPU alike (which
    step depends on rounding), so its comparison stops at 40 steps."""
    p, cfg = CASES[name]
    o = oracle_mod.Oracle(cfg, p)
    g = _sim(cfg, p)
    for _ in range(nsteps):
        assert o.step() == 0
    g.step(nsteps)
    # density of the final state: one more density evaluation on both sides
    o.step()
    g.step(1)
    ro, rg = o.get("rho"), g.get("rho")
    l1 = np.sum(np.abs(rg - ro)) / np.sum(np.abs(ro))
    assert l1 <= rtol, f"L1 {l1:.3e}"


@pytest.mark.parametrize("name", ["sedov16_periodic", "kh24"])
def test_link_modes_bitwise(name):
    """The face links in order, on a second stream beside the gradients, or
    inside the gradients kernel (link_overlap 0, 1, 2): the same face table
    and the same steps, bit for bit."""
    p, cfg = CASES[name]
    states, faces = [], []
    for lo in (0, 1, 2):
        sim = _sim(cfg, p)
        sim.set_tuning({"face_threads": 128, "face_blocks_per_sm": 4, "grad_threads": 64,
                        "nns_warps_per_sm": 32, "face_split": 1, "link_overlap": lo})
        st = sim.step(3)
        assert st.status == 0
        states.append(sim.get_state())
        faces.append(sim.get("face_of"))
        sim.close()
    for k in range(1, 3):
        assert np.array_equal(faces[0], faces[k])
        for key in states[0]:
            assert np.array_equal(states[0][key], states[k][key]), key
