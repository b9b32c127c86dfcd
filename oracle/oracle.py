"""TEST INFRASTRUCTURE (oracle): ctypes access to the CPU restatement
(oracle/libmlh_oracle.so) and to the reference build (oracle/_ref/ref_*).

Only tests/, the smoke check and bench.py's CPU baseline use this module, to
compare against; the product never imports it.
"""
from __future__ import annotations

import ctypes
import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libmlh_oracle.so")
# the same oracle computing in an operation-counting double (flop_count.hpp)
COUNT_LIB = os.path.join(HERE, "liborc_count.so")
REF_DIR = os.path.join(HERE, "_ref")

_INT_FIELDS = ["dim", "periodic", "adaptive_timestep", "slope_limiting", "pairwise_limiter",
               "meshless_finite_mass", "move_particles", "first_order_quad_point", "int_abs",
               "image_pairwise_limiter", "riemann_max_iter", "max_neighbours"]
_DBL_FIELDS = ["kernel_size", "gamma", "cfl", "time_step", "beta", "psi1", "psi2", "riemann_tol"]


class OrcConfig(ctypes.Structure):
    _fields_ = ([(f, ctypes.c_int) for f in _INT_FIELDS]
                + [("box_lo", ctypes.c_double * 3), ("box_hi", ctypes.c_double * 3)]
                + [(f, ctypes.c_double) for f in _DBL_FIELDS]
                + [("n_ngb", ctypes.c_double), ("adaptive_h", ctypes.c_int)])


INT_ARRAYS = {"noi", "noi_img", "off", "rev", "newton_iters", "nnl", "slot_iters"}


def reference_root() -> str:
    """The reference tree that oracle/build_ref.sh reads (MLH_REFERENCE, or
    the recipe's default); it exists only where the reference build runs."""
    r = subprocess.run(["bash", os.path.join(HERE, "build_ref.sh"), "--print-root"], capture_output=True,
                       text=True)
    return r.stdout.strip()


def build(counting: bool = False):
    subprocess.run(["make", "-s", "-C", HERE] + (["count"] if counting else []), check=True)


_libs = {}


def lib(counting: bool = False):
    """The oracle library (ctypes), or its operation-counting build."""
    if counting not in _libs:
        path = COUNT_LIB if counting else LIB
        build(counting)   # make: rebuilds a library older than its sources
        L = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [ctypes.POINTER(OrcConfig), ctypes.c_int] + [dp] * 8
        L.orc_step.restype = ctypes.c_int
        L.orc_step.argtypes = [ctypes.c_void_p]
        L.orc_size.restype = ctypes.c_long
        L.orc_size.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        L.orc_get.restype = ctypes.c_int
        L.orc_get.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p]
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        L.orc_riemann_batch.argtypes = [ctypes.c_int] + [dp] * 6 + [ctypes.c_double, dp, dp,
                                                                    ctypes.POINTER(ctypes.c_int)]
        L.orc_riemann_batch.restype = ctypes.c_int
        L.orc_riemann_fluxes.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 4 + [
            ctypes.c_double, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.orc_riemann_fluxes.restype = ctypes.c_int
        L.orc_smoothing_lengths.restype = ctypes.c_long
        L.orc_smoothing_lengths.argtypes = [ctypes.c_void_p, ctypes.c_double, dp, dp]
        L.orc_set_debug_level.restype = ctypes.c_int
        L.orc_set_debug_level.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_flux_asymmetric.restype = ctypes.c_long
        L.orc_flux_asymmetric.argtypes = [ctypes.c_void_p]
        L.orc_set_threads.restype = ctypes.c_int
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_flop_counts.restype = ctypes.c_int
        L.orc_flop_counts.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_ulonglong)]
        _libs[counting] = L
    return _libs[counting]


def set_threads(n: int) -> int:
    """Threads of the oracle's per-particle loops (n < 1: one per processor);
    the results do not depend on them.  Returns the count in effect."""
    return int(lib().orc_set_threads(int(n)))


def riemann_batch(rhoL, uL, pL, rhoR, uR, pR, gamma=5.0 / 3.0, guess=None):
    """Star pressure and Newton iterations of independent Riemann problems."""
    L = lib()
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (rhoL, uL, pL, rhoR, uR, pR)]
    n = arrs[0].size
    ps = np.zeros(n)
    it = np.zeros(n, dtype=np.int32)
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    g = None if guess is None else np.ascontiguousarray(guess, dtype=np.float64)
    L.orc_riemann_batch(n, *[dp(a) for a in arrs], gamma, None if g is None else dp(g), dp(ps),
                        it.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    return ps, it


def riemann_fluxes(Wi, Wj, vframe, aij, gamma=5.0 / 3.0, mfm=False):
    """Face fluxes of independent Riemann problems (Riemann::Riemann + exact)."""
    L = lib()
    Wi = np.ascontiguousarray(Wi, dtype=np.float64)
    Wj = np.ascontiguousarray(Wj, dtype=np.float64)
    vframe = np.ascontiguousarray(vframe, dtype=np.float64)
    aij = np.ascontiguousarray(aij, dtype=np.float64)
    n, nv = Wi.shape
    F = np.zeros((n, nv))
    it = np.zeros(n, dtype=np.int32)
    st = L.orc_riemann_fluxes(nv - 2, n, Wi.ctypes.data, Wj.ctypes.data, vframe.ctypes.data, aij.ctypes.data,
                              float(gamma), int(mfm), F.ctypes.data, it.ctypes.data)
    return F, it, st


def _cfg_struct(cfg) -> OrcConfig:
    s = OrcConfig()
    for f in _INT_FIELDS:
        setattr(s, f, int(getattr(cfg, f)))
    for a in range(3):
        s.box_lo[a] = float(cfg.box_lo[a])
        s.box_hi[a] = float(cfg.box_hi[a])
    for f in _DBL_FIELDS:
        setattr(s, f, float(getattr(cfg, f)))
    s.n_ngb = float(getattr(cfg, "n_ngb", 0.0))
    s.adaptive_h = int(getattr(cfg, "adaptive_h", False))
    return s


# stages of one step (ORC_STAGE_* in mlh_oracle.h) and the operation kinds
STAGES = ["binning", "hsolve", "nns", "density", "pressure", "timestep", "psi", "gradients", "limiter",
          "face", "states", "riemann", "collect", "update"]
OPS = ["add", "mul", "div", "sqrt", "pow", "fma"]


class Oracle:
    """One simulation held by the CPU restatement (counting=True: the
    operation-counting build, same results bit for bit)."""

    def __init__(self, cfg, pset, counting: bool = False):
        self.L = lib(counting)
        self._arrays = [np.ascontiguousarray(a, dtype=np.float64) for a in pset.arrays()]
        ptrs = [a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) for a in self._arrays]
        self._cfg = _cfg_struct(cfg)
        self.h = self.L.orc_create(ctypes.byref(self._cfg), pset.n, *ptrs)
        self.dim = cfg.dim

    def step(self) -> int:
        return self.L.orc_step(self.h)

    def set_debug_level(self, lvl: int):
        """The reference's DEBUG_LVL: 1 adds its checkFluxSymmetry to every step."""
        self.L.orc_set_debug_level(self.h, int(lvl))

    def flux_asymmetric(self) -> int:
        """Interactions checkFluxSymmetry found asymmetric in the last step."""
        return int(self.L.orc_flux_asymmetric(self.h))

    def get(self, name: str) -> np.ndarray:
        n = self.L.orc_size(self.h, name.encode())
        if n < 0:
            raise KeyError(name)
        if name in INT_ARRAYS:
            out = np.empty(n, dtype=np.uint32 if name == "nnl" else np.int32)
        else:
            out = np.empty(n, dtype=np.float64)
        if self.L.orc_get(self.h, name.encode(), out.ctypes.data) != 0:
            raise KeyError(name)
        return out

    def smoothing_lengths(self, n_ngb: float):
        """Per-particle smoothing lengths on the current positions: (h,
        effective neighbour number, number clamped at kernel_size)."""
        n = self.L.orc_size(self.h, b"x")
        h = np.empty(n)
        ne = np.empty(n)
        dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        clamped = self.L.orc_smoothing_lengths(self.h, float(n_ngb), dp(h), dp(ne))
        return h, ne, int(clamped)

    def flop_counts(self) -> dict:
        """Operation counts per stage summed over the steps so far
        ({stage: {op: count}}); counting build only."""
        out = (ctypes.c_ulonglong * (6 * len(STAGES)))()
        if self.L.orc_flop_counts(self.h, out) != len(STAGES):
            raise RuntimeError("not the operation-counting build of the oracle")
        return {st: {op: int(out[6 * k + q]) for q, op in enumerate(OPS)} for k, st in enumerate(STAGES)}

    def state(self) -> dict:
        names = ["x", "y", "vx", "vy", "m", "u"] + (["z", "vz"] if self.dim == 3 else [])
        return {k: self.get(k) for k in names}

    def close(self):
        if self.h:
            self.L.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- reference build

def read_dump(path: str) -> dict:
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    p = 0
    while p < len(data):
        (ln,) = struct.unpack_from("<I", data, p); p += 4
        name = data[p:p + ln].decode(); p += ln
        t = data[p:p + 1].decode(); p += 1
        (cnt,) = struct.unpack_from("<Q", data, p); p += 8
        dt = np.float64 if t == "d" else np.int32
        size = 8 if t == "d" else 4
        out[name] = np.frombuffer(data, dtype=dt, count=cnt, offset=p).copy()
        p += cnt * size
    if "nnl" in out:
        out["nnl"] = out["nnl"].view(np.uint32)
    return out


def ref_available(variant: str) -> bool:
    return os.path.exists(os.path.join(REF_DIR, "ref_" + variant))


def run_ref(variant: str, pset, nsteps: int, time_step: float = 0.005) -> dict:
    """Run the reference's own code (oracle/_ref/ref_<variant>) for nsteps."""
    exe = os.path.join(REF_DIR, "ref_" + variant)
    with tempfile.TemporaryDirectory() as td:
        fin = os.path.join(td, "in.bin")
        fout = os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            f.write(struct.pack("<q", pset.n))
            arrs = [pset.x, pset.y] + ([pset.z] if pset.dim == 3 else []) + \
                   [pset.vx, pset.vy] + ([pset.vz] if pset.dim == 3 else []) + [pset.m, pset.u]
            for a in arrs:
                f.write(np.ascontiguousarray(a, dtype=np.float64).tobytes())
        args = [exe, fin, fout, str(nsteps), repr(pset.kernel_size), repr(pset.gamma), repr(time_step)]
        args += [repr(float(v)) for v in pset.box_lo] + [repr(float(v)) for v in pset.box_hi]
        subprocess.run(args, check=True)
        return read_dump(fout)
