"""The learned p* guess: tensor-core MLP forward and gradients against the
float64 CPU reference (oracle/mlp_oracle.py), and GPU training on exact
Riemann solutions."""
import numpy as np
import pytest

from helpers import normwise

pytestmark = pytest.mark.gpu


def _features(rng, n):
    """Random left/right states and the network inputs for them."""
    rhoL = np.exp(rng.uniform(-2, 2, n)); rhoR = rhoL * np.exp(rng.uniform(-1.5, 1.5, n))
    pL = np.exp(rng.uniform(-6, 3, n)); pR = pL * np.exp(rng.uniform(-4, 4, n))
    g = 5.0 / 3.0
    cL = np.sqrt(g * pL / rhoL); cR = np.sqrt(g * pR / rhoR)
    uL = rng.normal(0, 0.5, n) * cL; uR = uL + rng.normal(0, 0.7, n) * cL
    x = np.stack([np.log(rhoR / rhoL), (uR - uL) / cL, np.log(pR / pL), np.log(cR / cL)], 1)
    return x.astype(np.float32), (rhoL, uL, pL, rhoR, uR, pR)


def test_forward_matches_cpu():
    import mlp_oracle
    from meshlesshydro_gb300 import build, runtime
    build.build()
    rng = np.random.default_rng(1)
    w = runtime.pstar_init(3)
    w[256:320] = rng.normal(0, 0.1, 64)       # nonzero biases exercise the bias path
    x, _ = _features(rng, 1000)
    y_gpu = runtime.pstar_infer(w, x)
    y_cpu, _ = mlp_oracle.forward(w, x)
    # BF16 activations between the layers: ~3 significant digits
    assert np.max(np.abs(y_gpu - y_cpu)) <= 2e-2 * (np.max(np.abs(y_cpu)) + 1e-3)


def test_gradient_matches_cpu():
    import mlp_oracle
    from meshlesshydro_gb300 import build, runtime
    build.build()
    rng = np.random.default_rng(2)
    w = runtime.pstar_init(5)
    x, _ = _features(rng, 1024)
    t = rng.normal(0, 1, 1024).astype(np.float32)
    loss_g, g_gpu = runtime.pstar_grad(w, x, t)
    loss_c, g_cpu = mlp_oracle.loss_and_grad(w, x, t)
    assert abs(loss_g - loss_c) <= 1e-2 * abs(loss_c)
    for name, (a, b) in mlp_oracle.SLICES.items():
        e = normwise(g_gpu[a:b], g_cpu[a:b])
        assert e <= 5e-2, f"{name}: normwise gradient error {e:.3e}"


def test_training_fits_exact_star_pressure(oracle_mod):
    from meshlesshydro_gb300 import build, runtime
    build.build()
    rng = np.random.default_rng(3)
    n = 65536
    x, (rhoL, uL, pL, rhoR, uR, pR) = _features(rng, n)
    ps, it_tr = oracle_mod.riemann_batch(rhoL, uL, pL, rhoR, uR, pR)
    t = np.log(ps / (0.5 * (pL + pR))).astype(np.float32)
    ok = np.isfinite(t) & (it_tr > 0)
    x, t = x[ok], t[ok]
    w, hist = runtime.pstar_train(x, t, epochs=12, batch=4096, lr=2e-3, seed=0)
    assert hist[-1] < 0.2 * hist[0], hist
    # the trained guess: Newton from p_mean * exp(y) converges, and the error
    # of the guess itself is far below that of the untrained network
    y = runtime.pstar_infer(w, x)
    rel_err = np.abs(np.exp(y - t) - 1.0)
    assert np.median(rel_err) < 0.05
