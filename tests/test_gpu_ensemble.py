"""Ensembles: many independent simulations of uneven sizes in one context.

Each member must evolve exactly as the same simulation run alone: neighbour
lists bit-exact (member-local indices), per-member dt, and fields within
FIELD_RTOL of the oracle run of that member.  Graph mode (one CUDA graph per
step) must give the same bits as direct launches.
"""
import numpy as np
import pytest

from meshlesshydro_gb300 import ic
from meshlesshydro_gb300.config import MFVConfig
from helpers import assert_close, assert_normwise

pytestmark = pytest.mark.gpu


def _members():
    return ic.kh_ensemble(n_members=5, seed=11, n_min=300, n_max=2000)


def _sim(cfg, members):
    from meshlesshydro_gb300 import build, runtime
    build.build()
    return runtime.Simulation(cfg, members=members)


def test_ensemble_members_match_single_runs(oracle_mod):
    members = _members()
    cfg = MFVConfig.kelvin_helmholtz(members[0])
    g = _sim(cfg, members)
    nsteps = 3
    g.step(nsteps)
    dt_g, t_g = g.member_times()
    state = g.get_state()
    first = 0
    for k, m in enumerate(members):
        o = oracle_mod.Oracle(MFVConfig.kelvin_helmholtz(m), m)
        t = 0.0
        for _ in range(nsteps):
            assert o.step() == 0
            t += o.get("dt")[0]
        assert_close([dt_g[k]], o.get("dt"), what=f"member {k} dt")
        assert_close([t_g[k]], [t], what=f"member {k} time")
        for key, v in o.state().items():
            assert_normwise(state[key][first:first + m.n], v, 1e-11, what=f"member {k} {key}")
        first += m.n


def test_ensemble_neighbour_lists(oracle_mod):
    members = _members()
    cfg = MFVConfig.kelvin_helmholtz(members[0])
    g = _sim(cfg, members)
    g.step(1)
    off = g.get("off")
    nnl = g.get("nnl")
    mask = (1 << 29) - 1
    first = 0
    for k, m in enumerate(members):
        o = oracle_mod.Oracle(MFVConfig.kelvin_helmholtz(m), m)
        o.step()
        lo, hi = off[first], off[first + m.n]
        mine = nnl[lo:hi]
        local = (mine & mask) - first
        assert local.min() >= 0 and local.max() < m.n
        recon = (mine & ~np.uint32(mask)) | local.astype(np.uint32)
        np.testing.assert_array_equal(recon, o.get("nnl"))
        np.testing.assert_array_equal(np.diff(off[first:first + m.n + 1]), np.diff(o.get("off")))
        first += m.n


def test_graph_mode_bitwise_equal():
    members = _members()
    cfg = MFVConfig.kelvin_helmholtz(members[0])
    a = _sim(cfg, members)
    b = _sim(cfg, members)
    b.set_graph_mode(True)
    a.step(4)
    st = b.step(4)
    assert st.steps == 4
    sa, sb = a.get_state(), b.get_state()
    for key in sa:
        assert np.array_equal(sa[key], sb[key]), key
    assert np.array_equal(a.member_times()[1], b.member_times()[1])


def test_graph_mode_single_sedov(oracle_mod):
    p = ic.sedov(n_side=12, seed=4, energy=0.05)
    cfg = MFVConfig.sedov(p, periodic=True)
    from meshlesshydro_gb300 import build, runtime
    build.build()
    g = runtime.Simulation(cfg, p)
    g.set_graph_mode(True)
    g.step(2)
    o = oracle_mod.Oracle(cfg, p)
    o.step(); o.step()
    gs = g.get_state()
    for key, v in o.state().items():
        assert_normwise(gs[key], v, 1e-11, what=key)


def test_autotune_keeps_results_bitwise():
    """The autotuner changes launch shapes only: the state after the tuning
    trials is restored, and later steps give the same bits."""
    members = _members()
    cfg = MFVConfig.kelvin_helmholtz(members[0])
    a = _sim(cfg, members)
    b = _sim(cfg, members)
    tuning = b.autotune(1)
    assert tuning["face_threads"] in (64, 128, 256)
    a.step(3)
    b.step(3)
    sa, sb = a.get_state(), b.get_state()
    for key in sa:
        assert np.array_equal(sa[key], sb[key]), key
    assert np.array_equal(a.member_times()[1], b.member_times()[1])


def test_set_tuning_validates_and_keeps_bits():
    from meshlesshydro_gb300 import runtime
    members = _members()
    cfg = MFVConfig.kelvin_helmholtz(members[0])
    a = _sim(cfg, members)
    b = _sim(cfg, members)
    c = _sim(cfg, members)
    b.set_tuning({"face_threads": 256, "face_blocks_per_sm": 3, "grad_threads": 64, "nns_warps_per_sm": 16})
    # the face links in order on the step's stream instead of beside the
    # time step and the gradients
    c.set_tuning({"face_threads": 128, "face_blocks_per_sm": 8, "grad_threads": 128, "nns_warps_per_sm": 64,
                  "link_overlap": 0})
    with pytest.raises(runtime.MLHError):
        b.set_tuning({"face_threads": 96, "face_blocks_per_sm": 3, "grad_threads": 64, "nns_warps_per_sm": 16})
    with pytest.raises(runtime.MLHError):
        b.set_tuning({"face_threads": 256, "face_blocks_per_sm": 3, "grad_threads": 64, "nns_warps_per_sm": 16,
                      "link_overlap": 3})
    for bad in ({"fp32_filters": 4}, {"fp32_filters": -1}, {"learned_guess": 2}, {"persistent_binning": 2}):
        with pytest.raises(runtime.MLHError):
            b.set_tuning(dict({"face_threads": 256, "face_blocks_per_sm": 3, "grad_threads": 64,
                               "nns_warps_per_sm": 16}, **bad))
    a.step(2)
    b.step(2)
    c.step(2)
    sa, sb, sc = a.get_state(), b.get_state(), c.get_state()
    for key in sa:
        assert np.array_equal(sa[key], sb[key]), key
        assert np.array_equal(sa[key], sc[key]), key
