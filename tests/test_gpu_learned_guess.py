"""The learned p* initial guess inside the step.

Strong shocks (p_TR > 2 min(pL, pR), p_TR the two-rarefaction guess) are
solved by Newton from p_TR * exp(y) where |y| > 0.01, y the network's output
(from p_TR elsewhere): inside the face block that holds them (the in-block
structure) or in a second pass around one batched network launch (the other
structures).  The converged p* satisfies
the same stopping rule as from the two-rarefaction guess, so the state must
stay on the oracle's trajectory within LEARNED_RTOL: the two Newton runs stop
at different points inside the tolerance band, which moves fluxes by
O(riemann_tol) relative.  A guess that does not converge restarts from the
two-rarefaction guess, so even a useless network gives correct results.
"""
import numpy as np
import pytest

from meshlesshydro_gb300 import ic
from meshlesshydro_gb300.config import MFVConfig
from helpers import assert_normwise

pytestmark = pytest.mark.gpu

# fields after a few steps, normwise relative (riemann_tol is 1e-10)
LEARNED_RTOL = 1e-9


def _runtime():
    from meshlesshydro_gb300 import build, runtime
    build.build()
    return runtime


def _cases():
    kh = ic.kelvin_helmholtz(n_side=40, seed=5)
    sd = ic.sedov(n_side=12, seed=4, energy=0.05)
    return [(MFVConfig.kelvin_helmholtz(kh), kh), (MFVConfig.sedov(sd, periodic=True), sd)]


@pytest.fixture(scope="module")
def trained():
    """Weights fitted to faces harvested from the two cases."""
    rt = _runtime()
    xs, ts = [], []
    for cfg, p in _cases():
        s = rt.Simulation(cfg, p)
        for _ in range(2):
            x, t = s.harvest(stride=1, capacity=1 << 20)
            xs.append(x); ts.append(t)
        s.close()
    x = np.concatenate(xs); t = np.concatenate(ts)
    w, hist = rt.pstar_train(x, t, epochs=40, batch=2048, lr=2e-3, seed=1)
    return w, hist, x, t


def test_harvest_records_faces():
    rt = _runtime()
    cfg, p = _cases()[0]
    s = rt.Simulation(cfg, p)
    ref = rt.Simulation(cfg, p)
    st = ref.step(1)
    x, t = s.harvest(stride=3, capacity=1 << 20)
    # every third canonical face with a converged solve
    assert abs(x.shape[0] - (st.faces + 2) // 3) <= 1
    assert np.all(np.isfinite(x)) and np.all(np.isfinite(t))
    # harvesting is one ordinary step
    a, b = s.get_state(), ref.get_state()
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_training_on_harvest(trained):
    w, hist, x, t = trained
    assert hist[-1] < 0.5 * hist[0], hist
    rt = _runtime()
    y = rt.pstar_infer(w, x)
    rel = np.abs(np.exp(y - t) - 1.0)
    assert np.median(rel) < 0.05, np.median(rel)


@pytest.mark.parametrize("case", [0, 1], ids=["kh40", "sedov12"])
def test_learned_guess_matches_oracle(trained, oracle_mod, case):
    w = trained[0]
    rt = _runtime()
    cfg, p = _cases()[case]
    s = rt.Simulation(cfg, p)
    s.set_pstar_weights(w)
    o = oracle_mod.Oracle(cfg, p)
    nsteps = 3
    st = s.step(nsteps)
    for _ in range(nsteps):
        assert o.step() == 0
    assert st.status == 0
    plain = rt.Simulation(cfg, p).step(nsteps)
    print(f"newton iterations per face: learned {st.newton_iterations / st.faces:.4f} "
          f"plain {plain.newton_iterations / plain.faces:.4f}; fallbacks {st.newton_fallbacks}; "
          f"learned faces {st.learned_faces} of {st.faces}")
    assert 0 <= st.learned_faces <= st.faces
    assert st.newton_fallbacks <= 0.01 * st.faces, (st.newton_fallbacks, st.faces)
    gs = s.get_state()
    for key, v in o.state().items():
        assert_normwise(gs[key], v, LEARNED_RTOL, what=key)


@pytest.mark.parametrize("case", [0, 1], ids=["kh40", "sedov12"])
def test_learned_face_structures_bitwise(trained, case):
    """With the learned guess, the structures of the first face pass (one
    pass; unfinished faces in a second pass over a queue; unfinished faces
    continued inside the block) defer the same strong shocks to the network
    and run the same arithmetic on every other face: identical states."""
    w = trained[0]
    rt = _runtime()
    cfg, p = _cases()[case]
    states = []
    for split in (0, 1, 2):
        s = rt.Simulation(cfg, p)
        s.set_tuning({"face_threads": 128, "face_blocks_per_sm": 4, "grad_threads": 64,
                      "nns_warps_per_sm": 32, "face_split": split})
        s.set_pstar_weights(w)
        s.step(3)
        states.append(s.get_state())
        s.close()
    for other in states[1:]:
        for k in states[0]:
            assert np.array_equal(states[0][k], other[k]), k


def test_bad_guess_falls_back(oracle_mod):
    """A network whose guess is e^20 times p_TR: Newton from there either
    converges or restarts from the two-rarefaction guess; the state stays on
    the oracle's trajectory either way."""
    rt = _runtime()
    cfg, p = _cases()[0]
    w = rt.pstar_init(2)
    w[-1] = 20.0            # output bias
    s = rt.Simulation(cfg, p)
    s.set_pstar_weights(w)
    o = oracle_mod.Oracle(cfg, p)
    st = s.step(2)
    o.step(); o.step()
    assert st.status == 0
    gs = s.get_state()
    for key, v in o.state().items():
        assert_normwise(gs[key], v, LEARNED_RTOL, what=key)


def test_learned_then_plain_graph_mode(trained):
    """Switching the guess on and off drops the captured graph; graph replay
    of the learned pipeline gives the bits of direct launches."""
    w = trained[0]
    rt = _runtime()
    cfg, p = _cases()[0]
    a = rt.Simulation(cfg, p)
    b = rt.Simulation(cfg, p)
    a.set_pstar_weights(w)
    b.set_pstar_weights(w)
    b.set_graph_mode(True)
    a.step(3); b.step(3)
    sa, sb = a.get_state(), b.get_state()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k
    a.set_pstar_weights(None)
    b.set_pstar_weights(None)
    a.step(1); b.step(1)
    sa, sb = a.get_state(), b.get_state()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k


@pytest.fixture(scope="module")
def strong_trained():
    """A network trained on faces harvested from the 24^3 Sedov blast (every
    face the learned step hands to the network in its first 30 steps, and
    every 8th face of its first step): a workload held out from the
    evaluation below."""
    rt = _runtime()
    p = ic.sedov(n_side=24, seed=4)
    s = rt.Simulation(MFVConfig.sedov(p, periodic=True), p)
    x, t = s.harvest(stride=8, capacity=1 << 20)
    xs, ts = [x], [t]
    for _ in range(30):
        x, t, _n = s.harvest(strong=True, capacity=1 << 20)
        xs.append(x); ts.append(t)
    s.close()
    x = np.concatenate(xs); t = np.concatenate(ts)
    w, hist = rt.pstar_train(x, t, epochs=60, batch=1024, lr=2e-3, seed=3)
    return w, x.shape[0]


def test_network_saves_newton_iterations_on_strong_shocks(strong_trained, oracle_mod):
    """What the trained network gains over the method without it, on a
    workload where the two-rarefaction guess is poor: 16 blasts in a 24^3
    periodic cube (ic.multi_blast; 4 or more Newton steps from p_TR on about
    5 % of the faces).  The learned step solves its strong shocks from the
    network's guess: fewer Newton steps than the plain step on the same three
    steps, with the fields of the oracle's trajectory (LEARNED_RTOL)."""
    w, nrows = strong_trained
    rt = _runtime()
    p = ic.multi_blast(n_side=24, n_blasts=16, seed=11)
    cfg = MFVConfig.sedov(p, periodic=True)
    plain = rt.Simulation(cfg, p)
    learned = rt.Simulation(cfg, p)
    learned.set_pstar_weights(w)
    a = plain.step(3)
    b = learned.step(3)
    assert a.status == 0 and b.status == 0
    assert a.faces == b.faces
    saved = a.newton_iterations - b.newton_iterations
    print(f"training rows {nrows}; faces {a.faces}; learned faces {b.learned_faces}; Newton steps plain "
          f"{a.newton_iterations} learned {b.newton_iterations}: {saved / max(b.learned_faces, 1):.2f} saved per "
          f"learned face; fallbacks {b.newton_fallbacks}")
    assert b.learned_faces >= 0.01 * b.faces
    assert b.newton_fallbacks <= 0.01 * b.learned_faces
    # fewer Newton steps with the network: at least 0.3 saved per face it guessed
    assert saved >= 0.3 * b.learned_faces, (saved, b.learned_faces)
    o = oracle_mod.Oracle(cfg, p)
    for _ in range(3):
        assert o.step() == 0
    ga, gb = plain.get_state(), learned.get_state()
    for key, v in o.state().items():
        assert_normwise(gb[key], v, LEARNED_RTOL, what="learned " + key)
        assert_normwise(gb[key], ga[key], LEARNED_RTOL, what="learned vs plain " + key)


def test_learned_guess_off_runs_the_plain_pipeline():
    """With weights set and mlh_tuning.learned_guess 0 (what the autotuner
    keeps where the network does not pay), the step is the plain step bit
    for bit and no face takes the network's guess; with 1 the network
    pipeline runs again."""
    rt = _runtime()
    cfg, p = _cases()[1]
    w = rt.pstar_init(7)
    base = {"face_threads": 128, "face_blocks_per_sm": 4, "grad_threads": 64, "nns_warps_per_sm": 32,
            "face_split": 1}
    plain = rt.Simulation(cfg, p)
    plain.set_tuning(base)
    st_p = plain.step(3)
    want = plain.get_state()
    plain.close()
    s = rt.Simulation(cfg, p)
    s.set_pstar_weights(w)
    s.set_tuning(dict(base, learned_guess=0))
    st = s.step(3)
    got = s.get_state()
    assert st.learned_faces == 0
    assert st.newton_iterations == st_p.newton_iterations
    for k in want:
        assert np.array_equal(got[k], want[k]), k
    s.set_tuning(dict(base, learned_guess=1))
    st = s.step(1)
    assert st.status == 0
    s.close()


def test_autotune_with_weights_picks_a_pipeline_and_restores_the_state():
    """With weights set the autotuner searches both face pipelines
    (learned_guess 1 and 0), reports the one it keeps, and leaves the state
    as it found it: the next steps are those of a context set to the
    reported tuning directly."""
    rt = _runtime()
    cfg, p = _cases()[1]
    w = rt.pstar_init(3)
    s = rt.Simulation(cfg, p)
    s.set_pstar_weights(w)
    before = s.get_state()
    tun = s.autotune(1)
    assert tun["learned_guess"] in (0, 1)
    after = s.get_state()
    for k in before:
        assert np.array_equal(before[k], after[k]), k
    st = s.step(2)
    assert st.status == 0
    got = s.get_state()
    s.close()
    ref = rt.Simulation(cfg, p)
    ref.set_pstar_weights(w)
    ref.set_tuning(tun)
    ref.step(2)
    want = ref.get_state()
    ref.close()
    for k in want:
        assert np.array_equal(got[k], want[k]), k
