"""Shared test helpers: fixture loading and tolerance checks."""
import os

import numpy as np

from meshlesshydro_gb300 import ic

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# Field tolerance of the parity tests, per element and per step (one step
# from identical inputs):
#     |a_i - b_i| <= FIELD_RTOL * max(|b_i|, scale_i)
# (b the oracle's value), where scale_i is the magnitude of the terms entry i
# is computed from, so that the gate is relative to what rounding can move:
#  * products and sums of positive terms (omega, rho, P, dt, m without mass
#    fluxes): scale 0, every entry to 1e-12 of its own value (measured
#    <= 9e-15 on every case; the 1e-5 background pressure of a Sedov blast is
#    held to 1e-12 of 1e-5);
#  * per-particle flux sums mF, eF, vF: sum_j max(|F_ij|, SUM_FLOOR max|F|)
#    of the component (the oracle's per-interaction fluxes, each with the
#    floor of the per-interaction gate below, so that a sum is held to what
#    its terms are held to); the new state: m, v, u from the update's terms
#    (|m v| + dt sum_j |F_p,ij|) / m_new and the like, x with |v| dt.  A
#    blast's pressure fluxes nearly cancel on every particle, so |vF| is a
#    small fraction of sum |F|: 1e-14 of the terms is 1e-12 of the sum and
#    more; in quiet regions the mass flux rho* (A . v*) is small against the
#    terms of u* = (uL + uR)/2 + (fR - fL)/2, which cancel;
#  * raw gradients, E^-1 and the per-interaction fluxes: SUM_FLOOR of the
#    field's largest magnitude (sums over neighbours whose terms cancel in
#    uniform regions);
#  * limited gradients: LIMITER_RTOL.  The limiter factor is the reference's
#    ratio (psi_max_ngb - psi_i) / (psi_max_mid - psi_i), whose differences are
#    1e-4 of psi_i in the nearly uniform background of a blast: a rounding of
#    psi_i moves the factor by 1e-12 relative and more.  The face states,
#    fluxes and new state of a particle whose limited gradient needs it, and
#    of its neighbours (the faces it shares), inherit it: LIMITER_RTOL there;
#  * ill-conditioned least-squares matrices: where a particle has few,
#    nearly coplanar neighbours (a blast's evacuated centre: 3 neighbours,
#    cond(E_i) = 1.2e8 after 63 steps of Sedov 64^3, against <= 2.7 for every
#    other particle), E_i^-1, its psi and gradients, the effective faces it
#    shares and so the fluxes and states of it and its neighbours move by
#    cond(E_i) ulp: those entries are held to COND_EPS * cond(E_i) (the
#    oracle's E_i^-1) where that exceeds the other tolerances;
#  * rank-deficient least-squares matrices: a particle with fewer than D
#    neighbours has a singular E_i (the sum of fewer than D outer products),
#    which the reference inverts all the same (the periodic Sedov 64^3
#    blast's evacuated centre, one neighbour at its 65th step, where the
#    reference's own update gives negative internal energy): E_i^-1 is
#    rounding noise in both codes, and so is everything computed from it.
#    Those particles and the particles they share faces with are left out
#    of the gate (limit infinity), counted, and the field scales are taken
#    over the others;
#  * Newton ties: faces whose iterations stop one step apart on the two sides
#    (the GPU's two-rarefaction guess and pressure functions use fifth roots,
#    reciprocals and reciprocal square roots a few ulp from the oracle's pow,
#    division and sqrt, so where the first step's change lies within that of
#    the 1e-10 stopping threshold, one side takes one more step; in that
#    quadratic regime the extra step moves p* by ~tol^2).  They are counted (at most
#    MAX_TIE_FRACTION of the faces) and the entries of their particles are
#    held to RIEMANN_TIE_RTOL.
# The normwise error max|a - b| / max|b| is reported beside it.  States after
# several steps, where differences compound, are compared normwise
# (assert_normwise) and by L1.
FIELD_RTOL = 1e-12
FIELD_FLOOR = 1e-3          # default floor of assert_close
SUM_FLOOR = 2e-2
LIMITER_RTOL = 1e-10
RIEMANN_TIE_RTOL = 1e-8
MAX_TIE_FRACTION = 1e-4
COND_EPS = 1e-15
COND_CAP = 1e-6             # the largest tolerance a condition number can give
EXACT_FIELDS = {"omega", "rho", "P", "dt"}


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


def assert_masked(a, b, floor, what, mask=None, rtol=FIELD_RTOL, rtol_masked=RIEMANN_TIE_RTOL, terms=None,
                  limits=None):
    """The per-element gate: |a - b| <= rtol * max(|b|, floor * max|b|,
    terms) (terms: the per-entry magnitude of the terms b is computed from,
    or None), entries under `mask` (Newton ties) held to rtol_masked; or,
    with `limits` (one tolerance per particle or slot, first axis), to
    those."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if b.size == 0:
        return
    scale = np.max(np.abs(b))
    den = np.maximum(np.abs(b), floor * scale)
    if terms is not None:
        den = np.maximum(den, np.asarray(terms, dtype=np.float64).reshape(b.shape))
    err = np.abs(a - b)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(err == 0.0, 0.0, err / den)
    lim = np.full(b.shape, rtol)
    if limits is not None:
        L = np.asarray(limits, dtype=np.float64)
        if b.ndim > 1:
            L = np.broadcast_to(L.reshape(-1, *([1] * (b.ndim - 1))), b.shape)
        lim = np.array(L, dtype=np.float64)
        excl = ~np.isfinite(lim)
        if excl.any():
            # entries left out of the gate: neither checked nor in the scale
            scale = np.max(np.abs(b[~excl]), initial=0.0)
            den = np.maximum(np.abs(b), floor * scale)
            if terms is not None:
                den = np.maximum(den, np.asarray(terms, dtype=np.float64).reshape(b.shape))
            with np.errstate(divide="ignore", invalid="ignore"):
                r = np.where(err == 0.0, 0.0, err / den)
            r[excl] = 0.0
    elif mask is not None:
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


def flux_terms(F, off, dim):
    """sum over each particle's interactions of max(|F_ij|, SUM_FLOOR
    max_kl |F_kl|) per flux component (N x (dim + 2)): the magnitude of the
    terms of its flux sums, each at least the floor the per-interaction gate
    allows it."""
    nv = dim + 2
    A = np.abs(np.asarray(F, dtype=np.float64).reshape(-1, nv))
    if A.size:
        A = np.maximum(A, SUM_FLOOR * A.max(axis=0, keepdims=True))
    cs = np.zeros((A.shape[0] + 1, nv))
    np.cumsum(A, axis=0, out=cs[1:])
    off = np.asarray(off, dtype=np.int64)
    return np.maximum(cs[off[1:]] - cs[off[:-1]], 0.0)


def state_terms(pre, post, S, dt, dim):
    """Per particle, the magnitude of the terms of the update
    (Particles::updateStateAndPosition, Particles.cpp:2013-2110) from the
    state `pre` to `post` with flux-term sums S (flux_terms) and time step dt:
    m from m and dt sum|F_m|; v from |m v| and dt sum|F_p| over the new mass;
    u from m (u + |v|^2/2) and dt sum|F_E| over the new mass plus |v_new|^2;
    x from |v| dt."""
    vk = ["vx", "vy", "vz"][:dim]
    m0 = np.abs(pre["m"])
    m1 = np.abs(post["m"])
    v0sq = sum(np.asarray(pre[k]) ** 2 for k in vk)
    v1sq = sum(np.asarray(post[k]) ** 2 for k in vk)
    out = {"m": m0 + dt * S[:, 0],
           "u": (m0 * (np.abs(pre["u"]) + 0.5 * v0sq) + dt * S[:, 1]) / m1 + v1sq}
    for a, k in enumerate(vk):
        out[k] = (m0 * np.abs(pre[k]) + dt * S[:, 2 + a]) / m1
    for k, v in zip("xyz"[:dim], vk):
        out[k] = np.abs(np.asarray(pre[v])) * dt
    return out


def assert_state(gs, ost, limits, what="", terms=None):
    """The state after one step from identical inputs, each entry relative to
    the magnitude of its update's terms (state_terms; without them a
    SUM_FLOOR floor for velocities), held to the particle's tolerance
    (step_limits; positions, which move with the old velocity, to
    FIELD_RTOL)."""
    for k, v in ost.items():
        t = None if terms is None else terms.get(k)
        floor = 0.0 if (t is not None or k in ("m", "u", "x", "y", "z")) else SUM_FLOOR
        lim = None if k in ("x", "y", "z") else limits
        assert_masked(gs[k], v, floor, what + "state " + k, terms=t, limits=lim)


def step_limits(g, o, dim):
    """Per-particle and per-slot tolerances of the entries downstream of the
    limiter and the face solve: FIELD_RTOL; LIMITER_RTOL for a particle whose
    limited gradient needs more than FIELD_RTOL (an ill-conditioned limiter
    factor) and for its neighbours; RIEMANN_TIE_RTOL for the particles of a
    Newton tie.  Returns (per-particle limits, per-slot limits, ties)."""
    off = np.asarray(o.get("off"), dtype=np.int64)
    n = off.size - 1
    nnl = np.asarray(o.get("nnl")).astype(np.int64) & ((1 << 29) - 1)
    owner = np.repeat(np.arange(n), np.diff(off))
    sens = np.zeros(n, dtype=bool)
    for f in ["rho", "vx", "vy"] + (["vz"] if dim == 3 else []) + ["P"]:
        a = np.asarray(g.get("grad_" + f), dtype=np.float64)
        b = np.asarray(o.get("grad_" + f), dtype=np.float64)
        den = np.maximum(np.abs(b), SUM_FLOOR * np.max(np.abs(b)))
        err = np.abs(a - b)
        with np.errstate(divide="ignore", invalid="ignore"):
            r = np.where(err == 0.0, 0.0, err / den)
        sens |= (r.reshape(n, 3) > FIELD_RTOL).any(axis=1)
    ring = sens.copy()
    ring[nnl[sens[owner]]] = True
    ring[owner[sens[nnl]]] = True
    tie, touched = riemann_ties(g, o)
    lim = np.full(n, FIELD_RTOL)
    lim[ring] = LIMITER_RTOL
    # cond(E_i) of the oracle's E_i^-1, spread to the particles that share a face
    B = np.asarray(o.get("B"), dtype=np.float64).reshape(n, dim, dim)
    cond = np.linalg.cond(B)
    cl = np.where(np.isfinite(cond), COND_EPS * cond, COND_CAP)
    slot_c = np.maximum(cl[owner], cl[nnl])
    cspread = cl.copy()
    np.maximum.at(cspread, owner, slot_c)
    lim = np.maximum(lim, np.minimum(cspread, COND_CAP))
    lim[touched] = np.maximum(lim[touched], RIEMANN_TIE_RTOL)
    # singular E_i (fewer than dim neighbours): out of the gate, with the
    # particles that share a face with it
    rank_def = rank_deficient(o, dim)
    if rank_def.any():
        out = rank_def.copy()
        out[nnl[rank_def[owner]]] = True
        out[owner[rank_def[nnl]]] = True
        lim[out] = np.inf
    slot = np.maximum(lim[owner], lim[nnl])
    slot[tie] = np.maximum(slot[tie], RIEMANN_TIE_RTOL)
    return lim, slot, tie


def rank_deficient(o, dim):
    """Particles with fewer than dim neighbours (images included): their
    least-squares matrix E_i is singular."""
    return (np.asarray(o.get("noi")) + np.asarray(o.get("noi_img"))) < dim


def compare_step(g, o, dim, slots=True, what="", pre=None):
    """One step of the GPU simulation g against the oracle o from identical
    inputs: neighbour lists and grid bit-exact; every stage array and the new
    state per element, with the scales and tolerances above (pre: the state
    the step started from, for the update's term scales).  slots=False skips
    the GPU's per-interaction flux array (large workloads compare its
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
    lim, slot_lim, tie = step_limits(g, o, dim)
    nfaces = max(int(o.get("stats")[0]), 1)
    assert tie.sum() / 2 <= MAX_TIE_FRACTION * nfaces + 1, f"{what}{tie.sum() // 2} Newton ties"
    nv = dim + 2
    Fo = o.get("F")
    if slots:
        assert_masked(g.get("F").reshape(-1, nv), Fo.reshape(-1, nv), SUM_FLOOR, what + "F", limits=slot_lim)
    S = flux_terms(Fo, o.get("off"), dim)
    del Fo
    for k, cols in (("mF", [0]), ("eF", [1]), ("vF", list(range(2, nv)))):
        a, b = g.get(k), o.get(k)
        if k == "vF":
            a = a.reshape(-1, 3)[:, :dim]
            b = b.reshape(-1, 3)[:, :dim]
        t = S[:, cols] if k == "vF" else S[:, cols[0]]
        assert_masked(a, b, 0.0, what + k, terms=t, limits=lim)
    ost = o.state()
    terms = state_terms(pre, ost, S, float(o.get("dt")[0]), dim) if pre is not None else None
    assert_state(g.get_state(), ost, lim, what, terms)
    return int(tie.sum() // 2)


def state_of(p):
    """The state arrays of particle set p (x, y, (z), vx, vy, (vz), m, u)."""
    keys = ["x", "y", "vx", "vy", "m", "u"] + (["z", "vz"] if p.dim == 3 else [])
    return {k: np.asarray(getattr(p, k)) for k in keys}


def pset_from_state(p, st):
    """A copy of particle set p with the state st (dict of x, y, (z), vx, vy,
    (vz), m, u arrays)."""
    q = p.copy()
    for k, v in st.items():
        setattr(q, k, np.ascontiguousarray(v, dtype=np.float64))
    return q
