"""Shared test helpers: fixture loading and tolerance checks."""
import os

import numpy as np

from meshlesshydro_gb300 import ic

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# Field tolerance of the parity tests, per element and per step (one step
# from identical inputs):
#     |a_i - b_i| <= FIELD_RTOL * max(|b_i|, FIELD_FLOOR * max_k |b_k|)
# (b the oracle's field).  Entries of at least FIELD_FLOOR of the field's
# largest magnitude are held to FIELD_RTOL of their own value; smaller ones
# to FIELD_RTOL * FIELD_FLOOR = 1e-15 of the field's largest magnitude.  The
# floor covers entries that are sums of terms far larger than themselves,
# which rounding leaves with absolute, not relative, errors of a few ulp of
# the terms: velocities that are zero up to rounding in the quiet region of a
# blast, gradients in uniform regions, coordinates near the origin.  (The
# reference build and the oracle, which differ only in the 2x2/3x3 inverse,
# already differ by 4.5e-17 of a field's maximum on a gradient entry
# 1.7e-6 of it.)  The normwise error max|a - b| / max|b| is reported beside it.
# States after several steps, where differences compound, are compared
# normwise (assert_normwise) and by L1.
FIELD_RTOL = 1e-12
FIELD_FLOOR = 1e-3


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def pset_from_golden(d):
    dim = int(d["dim"])
    return ic.ParticleSet(dim, d["in_x"], d["in_y"], d["in_z"], d["in_vx"], d["in_vy"], d["in_vz"],
                          d["in_m"], d["in_u"], float(d["kernel_size"]), tuple(d["box_lo"]),
                          tuple(d["box_hi"]), float(d["gamma"]))


def normwise(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if b.size == 0:
        return 0.0
    scale = np.max(np.abs(b))
    err = np.max(np.abs(a - b))
    return err / scale if scale > 0 else err


def elementwise(a, b, floor=FIELD_FLOOR):
    """max_i |a_i - b_i| / max(|b_i|, floor * max_k |b_k|), and the index i
    where it is reached (-1 for empty or all-zero fields that agree)."""
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    if b.size == 0:
        return 0.0, -1
    scale = np.max(np.abs(b))
    den = np.maximum(np.abs(b), floor * scale)
    diff = np.abs(a - b)
    if not np.all(np.isfinite(diff)):
        bad = int(np.nonzero(~np.isfinite(diff))[0][0])
        return float("inf"), bad
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(diff == 0.0, 0.0, diff / den)
    i = int(np.argmax(r))
    return float(r[i]), i


def assert_close(a, b, rtol=FIELD_RTOL, what="", floor=FIELD_FLOOR):
    """The per-element gate above; the message also gives the normwise error."""
    e, i = elementwise(a, b, floor)
    if not (np.isfinite(e) and e <= rtol):
        a = np.asarray(a, dtype=np.float64).ravel()
        b = np.asarray(b, dtype=np.float64).ravel()
        raise AssertionError(f"{what}: per-element relative error {e:.3e} > {rtol:.1e} at [{i}] "
                             f"(gpu {a[i]!r}, oracle {b[i]!r}, field max {np.max(np.abs(b)):.3e}); "
                             f"normwise {normwise(a, b):.3e}")


def assert_normwise(a, b, rtol, what=""):
    """max|a - b| <= rtol * max|b|: states after several steps."""
    e = normwise(a, b)
    assert np.isfinite(e) and e <= rtol, f"{what}: normwise relative error {e:.3e} > {rtol:.1e}"


def l1_rel(a, b):
    """sum |a - b| / sum |b|."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.sum(np.abs(a - b)) / np.sum(np.abs(b)))


def compare_step(g, o, dim, slots=True, what=""):
    """One step of the GPU simulation g against the oracle o from identical
    inputs: neighbour lists and grid bit-exact; density, pressure, dt,
    gradients (raw and limited), E^-1, fluxes and the new state per element
    (assert_close).  slots=False skips the per-interaction flux array (large
    workloads compare its per-particle sums instead)."""
    for k in ("off", "noi", "noi_img"):
        np.testing.assert_array_equal(g.get(k), o.get(k), err_msg=what + k)
    np.testing.assert_array_equal(g.get("nnl"), o.get("nnl"), err_msg=what + "nnl")
    np.testing.assert_array_equal(g.get("grid"), o.get("grid"), err_msg=what + "grid")
    for k in ("omega", "rho", "P", "dt"):
        assert_close(g.get(k), o.get(k), what=what + k)
    fields = ["rho", "vx", "vy"] + (["vz"] if dim == 3 else []) + ["P"]
    for f in fields:
        assert_close(g.get("gradraw_" + f), o.get("gradraw_" + f), what=what + "gradraw_" + f)
        assert_close(g.get("grad_" + f), o.get("grad_" + f), what=what + "grad_" + f)
    assert_close(g.get("B"), o.get("B"), what=what + "B")
    if slots:
        assert_close(g.get("F"), o.get("F"), what=what + "F")
    assert_close(g.get("mF"), o.get("mF"), what=what + "mF")
    assert_close(g.get("eF"), o.get("eF"), what=what + "eF")
    assert_close(g.get("vF").reshape(-1, 3)[:, :dim], o.get("vF").reshape(-1, 3)[:, :dim], what=what + "vF")
    gs = g.get_state()
    for k, v in o.state().items():
        assert_close(gs[k], v, what=what + "state " + k)


def pset_from_state(p, st):
    """A copy of particle set p with the state st (dict of x, y, (z), vx, vy,
    (vz), m, u arrays)."""
    q = p.copy()
    for k, v in st.items():
        setattr(q, k, np.ascontiguousarray(v, dtype=np.float64))
    return q
