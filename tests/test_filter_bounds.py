"""The error bounds of the single-precision filters (mlh_tuning.fp32_filters),
restated in numpy float32 and checked on the CPU over random and adversarial
inputs: the filters may only skip FP64 work whose result cannot matter.

* Slope limiter (k_gradients, Particles::slopeLimiter Particles.cpp:1313-1444):
  q_j = (c grad f) . (x_j - x_i) estimated in float32 from float32 positions;
  with B = 12 eps32 S R + 12 u64 (|f_i| + S R) + 1e-36 (S = sum |c grad f|,
  R = max|x| + max|x_j - x_i|), the neighbour holding the largest FP64
  f_ij = f_i + sum_a g_a d_a has q_j >= max_k q_k - 2 B (and the smallest
  q_j <= min_k q_k + 2 B).
* Time step (k_gradients' first pass, Particles::compGlobalTimestep
  Particles.cpp:1446-1485): the float32 signal speed vs_j = c_i + c_j +
  max(0, v_ij . (x_j - x_i) / r) is within B_j = 2 eps32 (2 (c_i + c_j) +
  2 vs_j + V (7 X / r + 8)) of the FP64 one (V = |v_i|_1 + |v_j|_1), so the
  float bounds on dt_i = cfl h / max_j vs_j bracket the FP64 dt_i.

The GPU side is checked bit for bit by tests/test_gpu_fp32_filters.py (the
same steps with the filters on and off); this file checks the arithmetic
argument itself.  numpy's float32 multiply-then-add rounds twice where the
kernels fuse: the bounds cover either.
"""
import numpy as np

EPS32 = np.float32(5.9604645e-8)
U64 = np.float32(1.1102230e-16)
f32 = np.float32


def _slope_case(rng, t, D):
    xi = rng.random(D)
    n = int(rng.integers(3, 64))
    if t % 3 == 0:   # lattice offsets: exact ties in the increments
        offs = rng.integers(-2, 3, size=(n, D)) * 0.01
    else:
        offs = (rng.random((n, D)) * 2 - 1) * 0.03
    xj = xi + offs
    # periodic wrap of the stored coordinate and its image back (unit box)
    wrapped = np.where(xj >= 1.0, xj - 1.0, np.where(xj < 0.0, xj + 1.0, xj))
    img = wrapped != xj
    ximg = np.where(img, np.where(wrapped < 0.5, 1.0 + wrapped, wrapped - 1.0), wrapped)
    d = ximg - xi
    g = rng.standard_normal(D) * 10.0 ** rng.integers(-12, 6)
    if t % 5 == 0:
        g[rng.integers(D)] = 0.0
    fi = rng.standard_normal() * 10.0 ** rng.integers(-6, 6)
    return xi, ximg, wrapped, img, d, g, fi


def test_slope_filter_window_holds_the_extrema():
    rng = np.random.default_rng(1)
    for D in (2, 3):
        for t in range(6000):
            xi, ximg, wrapped, img, d, g, fi = _slope_case(rng, t, D)
            if np.all(g == 0):
                continue
            fij = np.full(d.shape[0], fi)
            for a in range(D):
                fij = fij + g[a] * d[:, a]          # two roundings per step: no closer than the FMA chain
            gf = g.astype(f32)
            xif = xi.astype(f32)
            xjf = np.where(img, ximg.astype(f32), wrapped.astype(f32))
            df = (xjf - xif).astype(f32)
            q = (gf[0] * df[:, 0]).astype(f32)
            for a in range(1, D):
                q = (q + (gf[a] * df[:, a]).astype(f32)).astype(f32)
            R = f32(2.0) + f32(np.abs(df).max())    # |x| <= 1 in the box, + one box length for images
            S = f32(np.abs(gf).sum())
            B = f32(12) * EPS32 * S * R + f32(12) * U64 * (f32(abs(fi)) + S * R) + f32(1e-36)
            cand = (q >= q.max() - f32(2) * B) | (q <= q.min() + f32(2) * B)
            assert np.any(fij[cand] == fij.max()), (D, t)
            assert np.any(fij[cand] == fij.min()), (D, t)


def test_timestep_bounds_bracket_the_fp64_dt():
    rng = np.random.default_rng(2)
    for D in (2, 3):
        for t in range(4000):
            n = int(rng.integers(1, 40))
            xi = rng.random(D)
            xj = xi + (rng.random((n, D)) * 2 - 1) * 0.03
            xj = np.clip(xj, 0.0, 1.0)
            scale = 10.0 ** rng.integers(-3, 3)
            vi = rng.standard_normal(D) * scale
            vj = vi + rng.standard_normal((n, D)) * scale * (0.0 if t % 7 == 0 else 1.0)
            ci = abs(rng.standard_normal()) * scale + 1e-3
            cj = np.abs(rng.standard_normal(n)) * scale + 1e-3
            cfl_h = 0.3 * 0.02
            # FP64, as the exact kernel computes it
            dx = xj - xi
            r = np.sqrt(np.sum(dx * dx, axis=1))
            if np.any(r == 0):
                continue
            dv = np.sum((vi - vj) * (-dx), axis=1)
            vs = np.where(dv < 0, ci + cj - dv / r, ci + cj)
            dt64 = cfl_h / max(np.finfo(np.float64).tiny, vs.max())
            # float32 bounds, as k_gradients' first pass computes them
            xif, xjf = xi.astype(f32), xj.astype(f32)
            vif, vjf = vi.astype(f32), vj.astype(f32)
            d = (xjf - xif).astype(f32)
            w = (vif - vjf).astype(f32)
            dvd = np.sum((w * d).astype(f32), axis=1, dtype=f32)
            rf = np.sqrt(np.sum((d * d).astype(f32), axis=1, dtype=f32)).astype(f32)
            T = np.where(dvd > 0, (dvd / rf).astype(f32), f32(0))
            vsf = (f32(ci) + cj.astype(f32) + T).astype(f32)
            V = (np.abs(vif).sum() + np.abs(vjf).sum(axis=1)).astype(f32)
            X = f32(1.0)
            B = f32(2) * EPS32 * (f32(2) * (f32(ci) + cj.astype(f32)) + f32(2) * vsf
                                 + V * (f32(7) * X / rf + f32(8)))
            vlo = f32(max(0.0, (vsf - B).max()))
            vhi = f32((vsf + B).max())
            ch = f32(cfl_h)
            lo = np.nextafter(f32(ch / vhi), f32(0)) * (f32(1) - f32(4) * EPS32)
            assert lo <= dt64, (D, t)
            if vlo > 0:
                hi = np.nextafter(f32(ch / vlo), f32(np.inf)) * (f32(1) + f32(4) * EPS32)
                assert dt64 <= hi, (D, t)
