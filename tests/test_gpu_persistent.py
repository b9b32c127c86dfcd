"""The persistent binning (mlh_tuning.persistent_binning): the binning of a
step as one cooperative kernel whose phases wait on one another at grid
barriers.

* It gives the step of the launch-per-phase binning bit for bit, in direct
  launches and replayed from a CUDA graph, for single simulations and for an
  ensemble.
* Its waits are bounded: with the test hook that makes every barrier wait for
  one block more than the launch holds (a flag that nothing sets), the step
  gives up within the poll limit, reports MLH_ERR_TIMEOUT, completes no step
  and leaves the state untouched; with the hook off the context steps on as a
  fresh one would.
"""
import time

import numpy as np
import pytest

from meshlesshydro_gb300 import ic
from meshlesshydro_gb300.config import MFVConfig

pytestmark = pytest.mark.gpu

MLH_ERR_TIMEOUT = 1 << 11
BASE = {"face_threads": 128, "face_blocks_per_sm": 4, "grad_threads": 64, "nns_warps_per_sm": 32,
        "face_split": 1, "link_overlap": 1}


def _runtime():
    from meshlesshydro_gb300 import build, runtime
    build.build()
    return runtime


def _cases():
    kh = ic.kelvin_helmholtz(n_side=24, seed=3)
    sd = ic.sedov(n_side=16, seed=5)
    return {"kh24": (MFVConfig.kelvin_helmholtz(kh), kh, None),
            "sedov16_periodic": (MFVConfig.sedov(sd, periodic=True), sd, None),
            "sedov16_nonperiodic": (MFVConfig.sedov(sd, periodic=False), sd, None),
            "kh_ensemble8": (None, None, ic.kh_ensemble(n_members=8, seed=3, n_min=400, n_max=2500))}


def _make(rt, cfg, p, members):
    if members is not None:
        return rt.Simulation(MFVConfig.kelvin_helmholtz(members[0]), members=members)
    return rt.Simulation(cfg, p)


@pytest.mark.parametrize("name", sorted(_cases()))
@pytest.mark.parametrize("graph", [False, True], ids=["direct", "graph"])
def test_persistent_binning_gives_the_same_step(name, graph):
    rt = _runtime()
    cfg, p, members = _cases()[name]
    states = []
    for pb in (0, 1):
        s = _make(rt, cfg, p, members)
        s.set_tuning(dict(BASE, persistent_binning=pb))
        s.set_graph_mode(graph)
        st = s.step(3)
        assert st.steps == 3 and st.status == 0
        states.append((s.get_state(), s.get("nnl"), s.get("grid")))
        s.close()
    (a, na, ga), (b, nb, gb) = states
    assert np.array_equal(na, nb) and np.array_equal(ga, gb)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_barrier_timeout_is_reported_and_leaves_the_state():
    rt = _runtime()
    cfg, p, _ = _cases()["sedov16_periodic"]
    s = _make(rt, cfg, p, None)
    s.set_tuning(dict(BASE, persistent_binning=1))
    s.step(1)
    before = s.get_state()
    assert s.L.mlh_test_binning_barrier(s.h, 1, 2000) == 0
    t0 = time.perf_counter()
    st = s.step(1, check=False)
    elapsed = time.perf_counter() - t0
    assert st.status & MLH_ERR_TIMEOUT, st.status
    assert st.steps == 0
    assert elapsed < 10.0, elapsed
    after = s.get_state()
    for k in before:
        assert np.array_equal(before[k], after[k]), k
    # the hook off: the context steps on as a fresh one from the same state
    assert s.L.mlh_test_binning_barrier(s.h, 0, 0) == 0
    st = s.step(2)
    assert st.steps == 2 and st.status == 0
    ref = _make(rt, cfg, p, None)
    ref.set_tuning(dict(BASE, persistent_binning=1))
    ref.step(3)
    got, want = s.get_state(), ref.get_state()
    for k in got:
        assert np.array_equal(got[k], want[k]), k
