"""Shared test helpers: fixture loading and tolerance checks."""
import os

import numpy as np

from meshlesshydro_gb300 import ic

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# Field tolerance used throughout the parity tests: normwise relative error
# max_i |a_i - b_i| <= FIELD_RTOL * max_i |b_i| per field, per step.
FIELD_RTOL = 1e-12


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


def assert_close(a, b, rtol=FIELD_RTOL, what=""):
    e = normwise(a, b)
    assert np.isfinite(e) and e <= rtol, f"{what}: normwise relative error {e:.3e} > {rtol:.1e}"
