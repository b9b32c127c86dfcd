"""GPU parity of the per-particle smoothing lengths: mlh_smoothing_lengths and
adaptive_h steps (libmlh.so, through the C ABI) against the CPU oracle.

Bar: smoothing lengths and effective neighbour numbers bit-exact on identical
inputs (both sides perform the same explicitly rounded operations in the same
order), neighbour lists bit-exact, every other per-step field within the
per-element gate of helpers.assert_close; the adaptive steps start every
step from the oracle's state, so the smoothing lengths are compared bit for
bit at every step.  The oracle's solve is itself pinned against an
independent brute-force bisection by tests/test_oracle_hsolve.py.
"""
import numpy as np
import pytest

from meshlesshydro_gb300 import ic
from meshlesshydro_gb300.config import MFVConfig
from helpers import assert_close, compare_step, pset_from_state

pytestmark = pytest.mark.gpu


def _sim(cfg, p):
    from meshlesshydro_gb300 import build, runtime
    build.build()
    return runtime.Simulation(cfg, p)


def cases():
    kh = ic.kelvin_helmholtz(n_side=32, seed=3)
    sd = ic.sedov(n_side=14, seed=4, energy=0.05)
    return {
        "kh32": (kh, 20.0, MFVConfig.kelvin_helmholtz(kh, kernel_size=kh.kernel_size * 1.3)),
        "sedov14_periodic": (sd, 32.0, MFVConfig.sedov(sd, periodic=True, kernel_size=sd.kernel_size * 1.25)),
        "sedov14_nonperiodic": (sd, 32.0, MFVConfig.sedov(sd, periodic=False, kernel_size=sd.kernel_size * 1.25)),
    }


CASES = cases()


@pytest.mark.parametrize("name", sorted(CASES))
def test_smoothing_lengths_bitexact(oracle_mod, name):
    p, n_ngb, cfg = CASES[name]
    o = oracle_mod.Oracle(cfg, p)
    g = _sim(cfg, p)
    for target in (n_ngb, 1.4 * n_ngb, n_ngb):   # cold start, then warm starts up and down
        ho, neo, co = o.smoothing_lengths(target)
        hg, neg, cg = g.smoothing_lengths(target)
        np.testing.assert_array_equal(hg, ho)
        np.testing.assert_array_equal(neg, neo)
        assert cg == co
        free = hg < cfg.kernel_size
        assert np.max(np.abs(neg[free] - target)) <= 1e-11 * target
    g.close()


def test_smoothing_lengths_clamp_and_invalid(oracle_mod):
    p, _, cfg = CASES["kh32"]
    g = _sim(cfg, p)
    h, ne, clamped = g.smoothing_lengths(500.0)
    assert clamped == p.n and np.all(h == cfg.kernel_size)
    from meshlesshydro_gb300 import runtime
    with pytest.raises(runtime.MLHError):
        g.smoothing_lengths(5.0)   # below the particle's own count in 2D (40/7)
    g.close()


@pytest.mark.parametrize("name", sorted(CASES))
def test_adaptive_step_stagewise(oracle_mod, name):
    p, n_ngb, cfg0 = CASES[name]
    from dataclasses import replace
    cfg = replace(cfg0, adaptive_h=True, n_ngb=n_ngb)
    o = oracle_mod.Oracle(cfg, p)
    g = _sim(cfg, p)
    for step in range(3):
        # every step from the oracle's state (and both solves start from the
        # smoothing lengths of the previous step, equal bit for bit)
        pre = o.state()
        g.set_state(pset_from_state(p, pre))
        assert o.step() == 0
        st = g.step(1)
        assert st.steps == 1
        np.testing.assert_array_equal(g.get("h"), o.get("h"), err_msg=f"h, step {step}")
        compare_step(g, o, cfg.dim, slots=True, what=f"{name} step {step}: ", pre=pre)
    h = g.get("h")
    assert h.min() > 0 and h.max() <= cfg.kernel_size and h.std() > 0
    hs = g.get("h_stats")
    assert hs[0] >= p.n   # at least one iteration per particle
    g.close()


def test_uniform_lattice_gives_uniform_h(oracle_mod):
    """On an unjittered periodic lattice every particle sees the same
    neighbourhood: the solved h is uniform to rounding and N_eff hits the
    target (the sums run in a different order per particle)."""
    p = ic.kelvin_helmholtz(n_side=24, seed=3, jitter=0.0)
    cfg = MFVConfig.kelvin_helmholtz(p, kernel_size=p.kernel_size * 1.3)
    g = _sim(cfg, p)
    h, ne, clamped = g.smoothing_lengths(20.0)
    assert clamped == 0
    assert np.ptp(h) <= 1e-14 * h[0]
    assert np.max(np.abs(ne - 20.0)) <= 1e-11 * 20.0
    g.close()
