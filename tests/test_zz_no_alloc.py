"""The allocation-free grid-bounds entry point against the step's own grid.

mlh_grid_bounds_noalloc serves callers that cannot call cudaMalloc
(frameworks that own all device memory through their own pool, loops that
must not allocate after start-up); its scratch is a static device array.  This file is collected last so that a failure here leaves every other
test already run.  Each call is compared with the grid that mlh_step computed
from the same particle positions (exact equality, within FIELD_RTOL).
"""
import ctypes

import numpy as np
import pytest

from meshlesshydro_gb300 import ic
from meshlesshydro_gb300.config import MFVConfig
from helpers import assert_close

pytestmark = pytest.mark.gpu

MLH_ERR_CAPACITY = 1 << 23


def _call(L, torch, pos, dim, h, periodic=False, box=None):
    dev = torch.device("cuda")
    xs = [torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev) for a in pos]
    out = torch.full((9,), -1.0, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    lo = (ctypes.c_double * 3)(*(box[0] if box else (0, 0, 0)))
    hi = (ctypes.c_double * 3)(*(box[1] if box else (0, 0, 0)))
    z = xs[2].data_ptr() if dim == 3 else None
    rc = L.mlh_grid_bounds_noalloc(dim, 1 if periodic else 0, len(pos[0]), xs[0].data_ptr(), xs[1].data_ptr(), z,
                                   lo, hi, h, out.data_ptr(), None)
    return rc, out.cpu().numpy()


def test_noalloc_grid_matches_step_two_calls():
    torch = pytest.importorskip("torch")
    from meshlesshydro_gb300 import build, runtime
    build.build()
    L = runtime.load()
    grids = []
    # two calls in a row on different particle sets; each against the grid
    # the step computes for the same positions
    for n_side, seed in ((16, 5), (12, 9)):
        p = ic.sedov(n_side=n_side, seed=seed)
        sim = runtime.Simulation(MFVConfig.sedov(p, periodic=False), p)
        rc, grid = _call(L, torch, [p.x, p.y, p.z], 3, p.kernel_size)
        assert rc == 0, L.mlh_last_error()
        sim.step(1)
        assert_close(grid, sim.get("grid"), what=f"grid, {n_side}^3")
        # and from the moved positions the next step starts from
        st = sim.get_state()
        rc, grid_b = _call(L, torch, [st["x"], st["y"], st["z"]], 3, p.kernel_size)
        assert rc == 0, L.mlh_last_error()
        sim.step(1)
        assert_close(grid_b, sim.get("grid"), what=f"grid after one step, {n_side}^3")
        grids.append(grid)
    assert not np.array_equal(grids[0], grids[1])


def test_noalloc_periodic_2d_and_size_limit():
    torch = pytest.importorskip("torch")
    from meshlesshydro_gb300 import build, runtime
    build.build()
    L = runtime.load()
    p = ic.kelvin_helmholtz(n_side=24, seed=3)
    sim = runtime.Simulation(MFVConfig.kelvin_helmholtz(p), p)
    for _ in range(2):
        rc, grid = _call(L, torch, [p.x, p.y], 2, p.kernel_size, periodic=True, box=(p.box_lo, p.box_hi))
        assert rc == 0, L.mlh_last_error()
        sim.step(1)
        assert_close(grid, sim.get("grid"), what="periodic grid")
    # sizes beyond the stated maximum are rejected before any device work
    x = torch.zeros(4, dtype=torch.float64, device="cuda")
    out = torch.zeros(9, dtype=torch.float64, device="cuda")
    rc = L.mlh_grid_bounds_noalloc(2, 0, (1 << 29), x.data_ptr(), x.data_ptr(), None, None, None,
                                   0.1, out.data_ptr(), None)
    assert rc == MLH_ERR_CAPACITY
    assert b"MLH_NOALLOC_MAX_PARTICLES" in L.mlh_last_error()
    # a grid of more cells than an int counts is rejected with its own message
    q = ic.sedov(n_side=8, seed=2)
    rc, _ = _call(L, torch, [q.x, q.y, q.z], 3, 1e-4)
    assert rc & MLH_ERR_CAPACITY
    assert b"too many cells" in L.mlh_last_error()
