"""Shared test helpers: fixture loading and tolerance checks."""
import os

import numpy as np

from meshlesshydro_gb300 import ic

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# Field tolerance of the parity tests, per element and per step (one step
# from identical inputs):
#     |a_i - b_i| <= FIELD_RTOL * max(|b_i|, floor * max_k |b_k|)
# (b the oracle's field), with a floor per kind of field:
#  * products and sums of positive terms (omega, rho, P, dt, m, u and the
#    positions): no floor, every entry to 1e-12 of its own value (measured:
#    <= 9e-15 on every case; the 1e-5 background pressure of a Sedov blast is
#    held to 1e-12 of 1e-5);
#  * sums whose terms cancel (raw gradients, E^-1, face fluxes and their
#    per-particle sums, velocities): SUM_FLOOR of the field's largest
#    magnitude.  Their entries carry absolute errors of a few ulp of the terms
#    summed, not of the result: entries of at least SUM_FLOOR of the field's
#    maximum are held to 1e-12 of their own value, smaller ones to
#    1e-12 * SUM_FLOOR of the maximum.  (The reference build and the oracle,
#    which differ only in the 2x2/3x3 inverse, already differ by 4.5e-17 of a
#    field's maximum on a gradient entry 1.7e-6 of it.)
#  * limited gradients: LIMITER_RTOL.  The limiter factor is the reference's
#    ratio (psi_max_ngb - psi_i) / (psi_max_mid - psi_i), whose differences are
#    1e-4 of psi_i in the nearly uniform background of a blast: a rounding
#    of psi_i moves the factor by 1e-12 relative and more.
#  * a face where the two Newton iterations stop one step apart (the last
#    change of the one lands within rounding of the 1e-10 stopping
#    threshold; one face in ~10^6): p* then differs by up to the solver's
#    tolerance, and the fluxes and updated state of the face's two particles
#    are held to RIEMANN_TIE_RTOL (with the SUM_FLOOR floor); at most
#    MAX_TIE_FRACTION of the faces may be such ties.
# The normwise error max|a - b| / max|b| is reported beside it.  States after
# several steps, where differences compound, are compared normwise
# (assert_normwise) and by L1.
FIELD_RTOL = 1e-12
FIELD_FLOOR = 1e-3          # default floor of assert_close
SUM_FLOOR = 2e-2
LIMITER_RTOL = 1e-10
RIEMANN_TIE_RTOL = 1e-8
MAX_TIE_FRACTION = 1e-4
EXACT_FIELDS = {"omega", "rho", "P", "dt", "m", "u", "x", "y", "z"}


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


def riemann_ties(g, o):
    """Slots whose face took a different number of Newton steps on the GPU
    and in the oracle (boolean per slot), and the particles that own them."""
    gi = g.get("face_iters")
    oi = o.get("slot_iters")
    tie = gi != oi
    off = o.get("off")
    owner = np.repeat(np.arange(off.size - 1), np.diff(off))
    touched = np.zeros(off.size - 1, dtype=bool)
    touched[owner[tie]] = True
    return tie, touched


def assert_masked(a, b, floor, what, mask=None, rtol=FIELD_RTOL, rtol_masked=RIEMANN_TIE_RTOL):
    """The per-element gate with the field's own scale, entries under `mask`
    (Newton ties) held to rtol_masked instead of rtol."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if b.size == 0:
        return
    scale = np.max(np.abs(b))
    den = np.maximum(np.abs(b), floor * scale)
    err = np.abs(a - b)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(err == 0.0, 0.0, err / den)
    lim = np.full(b.shape, rtol)
    if mask is not None:
        m = np.asarray(mask, dtype=bool)
        if b.ndim > 1:
            m = np.broadcast_to(m.reshape(-1, *([1] * (b.ndim - 1))), b.shape)
        lim = np.where(m, rtol_masked, rtol)
    bad = ~(r <= lim)
    if bad.any():
        i = int(np.flatnonzero(bad.ravel())[0])
        raise AssertionError(f"{what}: per-element relative error {r.ravel()[i]:.3e} > {lim.ravel()[i]:.1e} at "
                             f"[{i}] (gpu {a.ravel()[i]!r}, oracle {b.ravel()[i]!r}, field max {scale:.3e}); "
                             f"{int(bad.sum())} entries; normwise {normwise(a, b):.3e}")


def assert_state(gs, ost, touched, what=""):
    """The state after one step from identical inputs: exact fields without a
    floor, velocities with SUM_FLOOR; the particles of a Newton tie to
    RIEMANN_TIE_RTOL (positions move with the old velocity: exact)."""
    for k, v in ost.items():
        floor = 0.0 if k in EXACT_FIELDS else SUM_FLOOR
        mask = None if k in ("x", "y", "z") else touched
        assert_masked(gs[k], v, floor, what + "state " + k, mask)


def compare_step(g, o, dim, slots=True, what=""):
    """One step of the GPU simulation g against the oracle o from identical
    inputs: neighbour lists and grid bit-exact; every stage array and the new
    state per element, with the floors and tolerances above.  slots=False
    skips the per-interaction flux array (large workloads compare its
    per-particle sums instead).  Returns the number of Newton ties."""
    for k in ("off", "noi", "noi_img"):
        np.testing.assert_array_equal(g.get(k), o.get(k), err_msg=what + k)
    np.testing.assert_array_equal(g.get("nnl"), o.get("nnl"), err_msg=what + "nnl")
    np.testing.assert_array_equal(g.get("grid"), o.get("grid"), err_msg=what + "grid")
    for k in ("omega", "rho", "P", "dt"):
        assert_close(g.get(k), o.get(k), floor=0.0, what=what + k)
    fields = ["rho", "vx", "vy"] + (["vz"] if dim == 3 else []) + ["P"]
    for f in fields:
        assert_close(g.get("gradraw_" + f), o.get("gradraw_" + f), floor=SUM_FLOOR, what=what + "gradraw_" + f)
        assert_close(g.get("grad_" + f), o.get("grad_" + f), rtol=LIMITER_RTOL, floor=SUM_FLOOR,
                     what=what + "grad_" + f)
    assert_close(g.get("B"), o.get("B"), floor=SUM_FLOOR, what=what + "B")
    tie, touched = riemann_ties(g, o)
    nfaces = max(int(o.get("stats")[0]), 1)
    assert tie.sum() / 2 <= MAX_TIE_FRACTION * nfaces + 1, f"{what}{tie.sum() // 2} Newton ties"
    if slots:
        nv = dim + 2
        assert_masked(g.get("F").reshape(-1, nv), o.get("F").reshape(-1, nv), SUM_FLOOR, what + "F", tie)
    for k in ("mF", "eF", "vF"):
        a, b = g.get(k), o.get(k)
        if k == "vF":
            a = a.reshape(-1, 3)[:, :dim]
            b = b.reshape(-1, 3)[:, :dim]
        assert_masked(a, b, SUM_FLOOR, what + k, touched)
    assert_state(g.get_state(), o.state(), touched, what)
    return int(tie.sum() // 2)


def pset_from_state(p, st):
    """A copy of particle set p with the state st (dict of x, y, (z), vx, vy,
    (vz), m, u arrays)."""
    q = p.copy()
    for k, v in st.items():
        setattr(q, k, np.ascontiguousarray(v, dtype=np.float64))
    return q
