"""Generate the golden fixtures of tests/golden/ from the reference's own code.

Runs the reference demonstrator's MFV stages, compiled unmodified from the
reference tree by oracle/build_ref.sh (oracle/_ref/ref_<variant>), on small
seeded inputs and stores inputs and outputs as .npz files.  The reference tree
is needed only here; the fixtures travel with the repository and pin the CPU
restatement (oracle/) on any host.

    python tests/golden/make_golden.py [name ...]   # after: bash oracle/build_ref.sh
                                                    # (no names: every fixture)

Variants (abs binding, see oracle/build_ref.sh):
  kh24_dbl      2D periodic Kelvin-Helmholtz, 24x24, fabs limiters
  kh24_int      same, limiters with the int abs(int) binding
  kh24pw_dbl    same set-up with PAIRWISE_LIMITER 1 (2D real faces)
  sedov12np_dbl 3D non-periodic Sedov 12^3 without the pairwise limiter (the
                reference's 3D pairwise limiter reads an uninitialised xjxi[2])
  kh100_dbl     the 100x100 Kelvin-Helmholtz set-up: lists and state after
                one step, state after ten steps
  kh24q_dbl     kh24pw_dbl with FIRST_ORDER_QUAD_POINT 0 (face point
                x_i + kernelSize/4 (x_j - x_i))
  sedov12q_dbl  3D non-periodic Sedov 12^3 with the pairwise limiter and
                FIRST_ORDER_QUAD_POINT 0, where the reference's 3D pairwise
                limiter reads only initialised values
  kh24mfm_dbl   kh24_dbl with MESHLESS_FINITE_MASS 1
  kh24fix_dbl   kh24_dbl with MOVE_PARTICLES 0
  kh24nolim_dbl kh24_dbl with SLOPE_LIMITING 0
  kh24pw_int    kh24pw_dbl with the int abs(int) binding (pairwise limiter,
                Particles.cpp:1748-1759, and slope limiter)
  kh24g14_dbl   kh24_dbl at gamma = 1.4 (set-up and configuration)
  sedov12g14_dbl sedov12np_dbl at gamma = 1.4
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from meshlesshydro_gb300 import ic  # noqa: E402
import oracle as O  # noqa: E402

STAGE_KEYS = ["off", "noi", "noi_img", "nnl", "omega", "rho", "P", "dt", "grid",
              "psi", "Aij", "vFrame", "WL", "WR", "F", "mF", "eF", "vF"]


def inputs(p):
    return {"in_x": p.x, "in_y": p.y, "in_z": p.z, "in_vx": p.vx, "in_vy": p.vy, "in_vz": p.vz,
            "in_m": p.m, "in_u": p.u, "kernel_size": np.array(p.kernel_size),
            "gamma": np.array(p.gamma), "box_lo": np.array(p.box_lo), "box_hi": np.array(p.box_hi),
            "dim": np.array(p.dim)}


SLOT_KEYS = {"psi": 1, "Aij": 1, "vFrame": 1, "WL": 2, "WR": 2, "F": 2}


def full(name, variant, p, nsteps, slot_particles=64):
    """Per-stage arrays of the first step; per-interaction arrays only for the
    slots of the first `slot_particles` particles (keeps the files small)."""
    r = O.run_ref(variant, p, nsteps)
    d = inputs(p)
    ns = int(r["off"][min(slot_particles, p.n)])
    for k in STAGE_KEYS:
        if k in SLOT_KEYS:
            width = p.dim if SLOT_KEYS[k] == 1 else p.dim + 2
            d[k] = r[k][: ns * width]
        else:
            d[k] = r[k]
    d["slot_particles"] = np.array(min(slot_particles, p.n))
    for k, v in r.items():
        if k.startswith(("grad_", "gradraw_", "s1_", "out_")) or k == "dts":
            d[k] = v
    d["nsteps"] = np.array(nsteps)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
    print("wrote", name, {k: v.shape for k, v in d.items() if hasattr(v, "shape") and v.size > 1})


def summary(name, variant, p, nsteps):
    r1 = O.run_ref(variant, p, 1)
    rn = O.run_ref(variant, p, nsteps)
    d = inputs(p)
    for k in ["off", "noi", "noi_img", "dt", "grid"]:
        d[k] = r1[k]
    d["nnl_sha256"] = np.frombuffer(hashlib.sha256(r1["nnl"].tobytes()).digest(), dtype=np.uint8)
    for k, v in r1.items():
        if k.startswith("s1_"):
            d[k] = v
    for k, v in rn.items():
        if k.startswith("out_") or k == "dts":
            d[k] = v
    d["nsteps"] = np.array(nsteps)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
    print("wrote", name)


def main(names):
    kh24 = lambda: ic.kelvin_helmholtz(n_side=24, seed=3)
    sd12 = lambda: ic.sedov(n_side=12, seed=4, energy=0.05)
    makers = {
        "kh24_dbl": lambda: full("kh24_dbl", "kh_dbl", kh24(), 5),
        "kh24_int": lambda: full("kh24_int", "kh_int", kh24(), 5),
        "kh24pw_dbl": lambda: full("kh24pw_dbl", "khpw_dbl", kh24(), 5),
        "sedov12np_dbl": lambda: full("sedov12np_dbl", "sedovnopw_dbl", sd12(), 1),
        "kh100_dbl": lambda: summary("kh100_dbl", "kh_dbl", ic.kelvin_helmholtz(n_side=100, seed=1), 10),
        "kh24q_dbl": lambda: full("kh24q_dbl", "khq_dbl", kh24(), 5),
        "sedov12q_dbl": lambda: full("sedov12q_dbl", "sedovq_dbl", sd12(), 1),
        "kh24mfm_dbl": lambda: full("kh24mfm_dbl", "khmfm_dbl", kh24(), 5),
        "kh24fix_dbl": lambda: full("kh24fix_dbl", "khfix_dbl", kh24(), 5),
        "kh24nolim_dbl": lambda: full("kh24nolim_dbl", "khnolim_dbl", kh24(), 5),
        "kh24pw_int": lambda: full("kh24pw_int", "khpw_int", kh24(), 5),
        "kh24g14_dbl": lambda: full("kh24g14_dbl", "kh_dbl", ic.kelvin_helmholtz(n_side=24, seed=3, gamma=1.4), 5),
        "sedov12g14_dbl": lambda: full("sedov12g14_dbl", "sedovnopw_dbl",
                                       ic.sedov(n_side=12, seed=4, energy=0.05, gamma=1.4), 1),
    }
    for name in names or list(makers):
        makers[name]()


if __name__ == "__main__":
    main(sys.argv[1:])
