"""ctypes binding of the C ABI in include/mlh.h (libmlh.so).

`Simulation` is the Python face of one mlh context: the reference's
MeshlessScheme driving one Particles set (demonstrator/src/MeshlessScheme.cpp:8-19
for construction, :39-253 for a step).  There is no CPU fallback: loading
fails loudly when the CUDA library is missing or no GPU is visible.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .config import CConfig, MFVConfig, to_struct

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmlh.so")

ERR_BITS = {
    0: "NGB_OVERFLOW", 1: "NEG_PRESSURE", 2: "NEG_DENSITY", 3: "NEG_MASS", 4: "NEG_ENERGY",
    5: "NEWTON", 6: "VACUUM", 7: "GRID", 8: "NO_NEIGHBOUR", 9: "ASYMMETRIC", 10: "NAN",
    11: "TIMEOUT", 20: "INVALID", 21: "CUDA", 22: "NO_DEVICE", 23: "CAPACITY",
}


def status_names(st: int):
    return [name for bit, name in ERR_BITS.items() if st & (1 << bit)]


class MLHError(RuntimeError):
    def __init__(self, status: int, where: str, msg: str = ""):
        super().__init__(f"{where}: status {status:#x} {status_names(status)} {msg}")
        self.status = status


class MemberDesc(ctypes.Structure):
    """mlh_member: one simulation of an ensemble."""
    _fields_ = [("n", ctypes.c_int), ("kernel_size", ctypes.c_double),
                ("box_lo", ctypes.c_double * 3), ("box_hi", ctypes.c_double * 3)]


class Tuning(ctypes.Structure):
    """mlh_tuning: launch shapes chosen by the autotuner."""
    _fields_ = [("face_threads", ctypes.c_int), ("face_blocks_per_sm", ctypes.c_int),
                ("grad_threads", ctypes.c_int), ("nns_warps_per_sm", ctypes.c_int),
                ("face_split", ctypes.c_int),
                ("link_overlap", ctypes.c_int), ("persistent_binning", ctypes.c_int),
                ("fp32_filters", ctypes.c_int), ("learned_guess", ctypes.c_int)]


class ParticlesView(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int)] + [(k, ctypes.POINTER(ctypes.c_double))
                                         for k in ("x", "y", "z", "vx", "vy", "vz", "m", "u")]


class StepStats(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int), ("status", ctypes.c_uint), ("dt", ctypes.c_double),
                ("time", ctypes.c_double), ("pair_interactions", ctypes.c_longlong),
                ("faces", ctypes.c_longlong), ("newton_iterations", ctypes.c_longlong),
                ("device_ms", ctypes.c_double), ("newton_fallbacks", ctypes.c_longlong),
                ("learned_faces", ctypes.c_longlong)]


EXPORTS = ["mlh_abi_version", "mlh_last_error", "mlh_create", "mlh_destroy", "mlh_set_fields",
           "mlh_get_fields", "mlh_step", "mlh_stage_array", "mlh_set_kernel_timing",
           "mlh_kernel_times", "mlh_reset_kernel_times", "mlh_probe_fp64_tflops", "mlh_probe_fp64_clock",
           "mlh_grid_bounds_noalloc", "mlh_ensemble_create", "mlh_member_times", "mlh_set_graph_mode",
           "mlh_autotune", "mlh_set_tuning", "mlh_pstar_infer", "mlh_pstar_grad", "mlh_pstar_train", "mlh_set_pstar_weights",
           "mlh_pstar_harvest", "mlh_pstar_harvest_strong", "mlh_smoothing_lengths", "mlh_prepare", "mlh_riemann_fluxes",
           "mlh_probe_fast_math", "mlh_probe_scale2", "mlh_probe_fp64_lanes", "mlh_test_binning_barrier"]

_lib = None


def load(path: str = LIB_PATH):
    """Load libmlh.so and declare the C ABI.  Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with meshlesshydro_gb300.build.build()")
    L = ctypes.CDLL(path)
    vp = ctypes.c_void_p
    L.mlh_abi_version.restype = ctypes.c_int
    L.mlh_last_error.restype = ctypes.c_char_p
    L.mlh_create.argtypes = [ctypes.POINTER(CConfig), ctypes.POINTER(ParticlesView), ctypes.POINTER(vp)]
    L.mlh_create.restype = ctypes.c_int
    L.mlh_destroy.argtypes = [vp]
    L.mlh_set_fields.argtypes = [vp, ctypes.POINTER(ParticlesView)]
    L.mlh_set_fields.restype = ctypes.c_int
    L.mlh_get_fields.argtypes = [vp, ctypes.POINTER(ParticlesView)]
    L.mlh_get_fields.restype = ctypes.c_int
    L.mlh_step.argtypes = [vp, ctypes.c_int, ctypes.c_double, ctypes.POINTER(StepStats)]
    L.mlh_step.restype = ctypes.c_int
    L.mlh_stage_array.argtypes = [vp, ctypes.c_char_p, vp, ctypes.c_longlong, ctypes.POINTER(ctypes.c_longlong)]
    L.mlh_stage_array.restype = ctypes.c_int
    L.mlh_set_kernel_timing.argtypes = [vp, ctypes.c_int]
    L.mlh_set_kernel_timing.restype = ctypes.c_int
    L.mlh_kernel_times.argtypes = [vp, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(ctypes.c_longlong),
                                   ctypes.POINTER(ctypes.c_double), ctypes.c_int]
    L.mlh_kernel_times.restype = ctypes.c_int
    L.mlh_reset_kernel_times.argtypes = [vp]
    L.mlh_probe_fp64_tflops.argtypes = [ctypes.c_double, ctypes.POINTER(ctypes.c_double)]
    L.mlh_probe_fp64_tflops.restype = ctypes.c_int
    L.mlh_probe_fp64_clock.argtypes = [ctypes.c_double, ctypes.POINTER(ctypes.c_double),
                                       ctypes.POINTER(ctypes.c_double)]
    L.mlh_test_binning_barrier.argtypes = [ctypes.c_void_p, ctypes.c_uint, ctypes.c_uint]
    L.mlh_test_binning_barrier.restype = ctypes.c_int
    L.mlh_probe_fp64_clock.restype = ctypes.c_int
    dp = ctypes.c_void_p
    L.mlh_grid_bounds_noalloc.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp, dp,
                                          ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                          ctypes.c_double, dp, dp]
    L.mlh_grid_bounds_noalloc.restype = ctypes.c_int
    L.mlh_ensemble_create.argtypes = [ctypes.POINTER(CConfig), ctypes.c_int, ctypes.POINTER(MemberDesc),
                                      ctypes.POINTER(ParticlesView), ctypes.POINTER(vp)]
    L.mlh_ensemble_create.restype = ctypes.c_int
    L.mlh_member_times.argtypes = [vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.c_int]
    L.mlh_member_times.restype = ctypes.c_int
    L.mlh_set_graph_mode.argtypes = [vp, ctypes.c_int]
    L.mlh_set_graph_mode.restype = ctypes.c_int
    L.mlh_autotune.argtypes = [vp, ctypes.c_int, ctypes.POINTER(Tuning)]
    L.mlh_autotune.restype = ctypes.c_int
    L.mlh_set_tuning.argtypes = [vp, ctypes.POINTER(Tuning)]
    L.mlh_set_tuning.restype = ctypes.c_int
    fp = ctypes.POINTER(ctypes.c_float)
    L.mlh_pstar_infer.argtypes = [fp, fp, ctypes.c_int, fp]
    L.mlh_pstar_infer.restype = ctypes.c_int
    L.mlh_pstar_grad.argtypes = [fp, fp, fp, ctypes.c_int, fp, fp]
    L.mlh_pstar_grad.restype = ctypes.c_int
    L.mlh_pstar_train.argtypes = [fp, fp, ctypes.c_longlong, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                  ctypes.c_uint, fp, fp]
    L.mlh_pstar_train.restype = ctypes.c_int
    L.mlh_set_pstar_weights.argtypes = [vp, fp]
    L.mlh_set_pstar_weights.restype = ctypes.c_int
    L.mlh_pstar_harvest.argtypes = [vp, ctypes.c_int, fp, fp, ctypes.c_longlong, ctypes.POINTER(ctypes.c_longlong)]
    L.mlh_pstar_harvest.restype = ctypes.c_int
    L.mlh_pstar_harvest_strong.argtypes = [vp, fp, fp, ctypes.c_longlong, ctypes.POINTER(ctypes.c_longlong)]
    L.mlh_pstar_harvest_strong.restype = ctypes.c_int
    L.mlh_smoothing_lengths.argtypes = [vp, ctypes.c_double, ctypes.POINTER(ctypes.c_double),
                                        ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong)]
    L.mlh_smoothing_lengths.restype = ctypes.c_int
    L.mlh_prepare.argtypes = [vp, ctypes.c_double]
    L.mlh_prepare.restype = ctypes.c_int
    L.mlh_riemann_fluxes.argtypes = [ctypes.c_int, ctypes.c_int] + [dp] * 4 + [ctypes.c_double, ctypes.c_int, dp, dp]
    L.mlh_riemann_fluxes.restype = ctypes.c_int
    L.mlh_probe_fast_math.argtypes = [ctypes.c_int] + [dp] * 5
    L.mlh_probe_fast_math.restype = ctypes.c_int
    L.mlh_probe_scale2.argtypes = [ctypes.c_int] + [dp] * 4
    L.mlh_probe_scale2.restype = ctypes.c_int
    L.mlh_probe_fp64_lanes.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    L.mlh_probe_fp64_lanes.restype = ctypes.c_int
    _lib = L
    return L


INT_ARRAYS = {"noi", "noi_img", "off", "nnl", "face_of", "face_iters"}


class HostState:
    """Pinned-free host SoA buffers matching mlh_particles_view."""

    def __init__(self, pset=None, n=None, dim=None):
        if pset is not None:
            self.n, self.dim = pset.n, pset.dim
            self.arrays = {k: np.ascontiguousarray(a, dtype=np.float64).copy()
                           for k, a in zip(("x", "y", "z", "vx", "vy", "vz", "m", "u"), pset.arrays())}
        else:
            self.n, self.dim = n, dim
            self.arrays = {k: np.zeros(n) for k in ("x", "y", "z", "vx", "vy", "vz", "m", "u")}
        self.view = ParticlesView()
        self.view.n = self.n
        for k, a in self.arrays.items():
            setattr(self.view, k, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))


def probe_fp64_tflops(seconds: float = 0.5) -> float:
    """FP64 FMA throughput of the current GPU in TFLOP/s (mlh_probe_fp64_tflops)."""
    L = load()
    out = ctypes.c_double()
    st = L.mlh_probe_fp64_tflops(seconds, ctypes.byref(out))
    if st != 0:
        raise MLHError(st, "mlh_probe_fp64_tflops", L.mlh_last_error().decode())
    return out.value


def probe_fp64_clock(seconds: float = 0.5):
    """(TFLOP/s, effective SM clock in MHz) of the FP64 FMA probe
    (mlh_probe_fp64_clock)."""
    L = load()
    tf = ctypes.c_double()
    mhz = ctypes.c_double()
    st = L.mlh_probe_fp64_clock(seconds, ctypes.byref(tf), ctypes.byref(mhz))
    if st != 0:
        raise MLHError(st, "mlh_probe_fp64_clock", L.mlh_last_error().decode())
    return tf.value, mhz.value


def probe_fp64_lanes(active_lanes: int, iters: int = 2048) -> float:
    """Device ms of the FP64 FMA chains run by only `active_lanes` lanes of
    every warp (mlh_probe_fp64_lanes)."""
    L = load()
    out = ctypes.c_double()
    st = L.mlh_probe_fp64_lanes(active_lanes, iters, ctypes.byref(out))
    if st != 0:
        raise MLHError(st, "mlh_probe_fp64_lanes", L.mlh_last_error().decode())
    return out.value


PSTAR_PARAMS = 8705


def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def pstar_init(seed: int = 0) -> np.ndarray:
    """Initial MLP parameters (Glorot-uniform weights, zero biases)."""
    rng = np.random.default_rng(seed)
    parts = []
    for fan_in, fan_out in ((4, 64), (64, 64), (64, 64), (64, 1)):
        lim = np.sqrt(6.0 / (fan_in + fan_out))
        parts.append(rng.uniform(-lim, lim, fan_out * fan_in))
        parts.append(np.zeros(fan_out))
    w = np.concatenate(parts).astype(np.float32)
    assert w.size == PSTAR_PARAMS
    return w


def pstar_infer(weights, x) -> np.ndarray:
    L = load()
    w = np.ascontiguousarray(weights, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, 4)
    y = np.empty(x.shape[0], dtype=np.float32)
    st = L.mlh_pstar_infer(_fptr(w), _fptr(x), x.shape[0], _fptr(y))
    if st != 0:
        raise MLHError(st, "mlh_pstar_infer", L.mlh_last_error().decode())
    return y


def pstar_grad(weights, x, t):
    L = load()
    w = np.ascontiguousarray(weights, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, 4)
    t = np.ascontiguousarray(t, dtype=np.float32)
    loss = np.zeros(1, dtype=np.float32)
    g = np.zeros(PSTAR_PARAMS, dtype=np.float32)
    st = L.mlh_pstar_grad(_fptr(w), _fptr(x), _fptr(t), x.shape[0], _fptr(loss), _fptr(g))
    if st != 0:
        raise MLHError(st, "mlh_pstar_grad", L.mlh_last_error().decode())
    return float(loss[0]), g


def pstar_train(x, t, weights=None, epochs: int = 10, batch: int = 4096, lr: float = 1e-3, seed: int = 0):
    L = load()
    w = np.ascontiguousarray(pstar_init(seed) if weights is None else weights, dtype=np.float32).copy()
    x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1, 4)
    t = np.ascontiguousarray(t, dtype=np.float32)
    hist = np.zeros(epochs, dtype=np.float32)
    st = L.mlh_pstar_train(_fptr(x), _fptr(t), x.shape[0], epochs, batch, lr, seed, _fptr(w), _fptr(hist))
    if st != 0:
        raise MLHError(st, "mlh_pstar_train", L.mlh_last_error().decode())
    return w, hist


def riemann_fluxes(Wi, Wj, vframe, aij, gamma: float = 5.0 / 3.0, mfm: bool = False):
    """Face fluxes of independent Riemann problems on the GPU (mlh_riemann_fluxes).
    Wi (left, particle i), Wj (right): (n, dim + 2) [rho, P, v...]; vframe, aij: (n, dim).
    Returns (F (n, dim + 2) [mass, energy, momentum], Newton iterations, status)."""
    L = load()
    Wi = np.ascontiguousarray(Wi, dtype=np.float64)
    Wj = np.ascontiguousarray(Wj, dtype=np.float64)
    vframe = np.ascontiguousarray(vframe, dtype=np.float64)
    aij = np.ascontiguousarray(aij, dtype=np.float64)
    n, nv = Wi.shape
    dim = nv - 2
    F = np.zeros((n, nv))
    it = np.zeros(n, dtype=np.int32)
    st = L.mlh_riemann_fluxes(dim, n, Wi.ctypes.data, Wj.ctypes.data, vframe.ctypes.data, aij.ctypes.data,
                              float(gamma), int(mfm), F.ctypes.data, it.ctypes.data)
    if st & ((1 << 20) | (1 << 21) | (1 << 22)):
        raise MLHError(st, "mlh_riemann_fluxes", L.mlh_last_error().decode())
    return F, it, st


class Simulation:
    """One MFV simulation on the GPU through the C ABI.

    With `members` (a list of ParticleSets) the context is an ensemble of
    independent simulations stored back to back (mlh_ensemble_create); `pset`
    is then ignored and the state arrays are the concatenation.
    """

    def __init__(self, cfg: MFVConfig, pset=None, members=None):
        if pset is None and not members:
            raise ValueError("Simulation needs a particle set or a list of members")
        self.L = load()
        self.cfg = cfg
        self._cfg = to_struct(cfg)
        self.dim = cfg.dim
        h = ctypes.c_void_p()
        if members is None:
            self.host = HostState(pset)
            self.n = pset.n
            self.nmembers = 1
            st = self.L.mlh_create(ctypes.byref(self._cfg), ctypes.byref(self.host.view), ctypes.byref(h))
            where = "mlh_create"
        else:
            from .ic import concatenate
            allp = concatenate(members)
            self.host = HostState(allp)
            self.n = allp.n
            self.nmembers = len(members)
            self.member_sizes = [m.n for m in members]
            descs = (MemberDesc * len(members))()
            for k, m in enumerate(members):
                descs[k].n = m.n
                descs[k].kernel_size = m.kernel_size
                for a in range(3):
                    descs[k].box_lo[a] = float(m.box_lo[a])
                    descs[k].box_hi[a] = float(m.box_hi[a])
            st = self.L.mlh_ensemble_create(ctypes.byref(self._cfg), len(members), descs,
                                            ctypes.byref(self.host.view), ctypes.byref(h))
            where = "mlh_ensemble_create"
        if st != 0:
            raise MLHError(st, where, self.L.mlh_last_error().decode())
        self.h = h

    def member_times(self):
        dt = np.zeros(self.nmembers)
        t = np.zeros(self.nmembers)
        st = self.L.mlh_member_times(self.h, dt.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                     t.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), self.nmembers)
        if st != 0:
            raise MLHError(st, "mlh_member_times", self.L.mlh_last_error().decode())
        return dt, t

    def set_graph_mode(self, on: bool):
        self.L.mlh_set_graph_mode(self.h, 1 if on else 0)

    def set_pstar_weights(self, weights):
        """Learned initial guess for the Riemann solves (None: two-rarefaction)."""
        self._pstar_w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float32)
        st = self.L.mlh_set_pstar_weights(self.h, None if weights is None else _fptr(self._pstar_w))
        if st != 0:
            raise MLHError(st, "mlh_set_pstar_weights", self.L.mlh_last_error().decode())

    def harvest(self, stride: int = 1, capacity: int = 1 << 22, strong: bool = False, check: bool = True):
        """One step recording (network input, log(p*/p_TR)) of every stride-th face,
        p_TR the two-rarefaction guess of the face; strong=True: of every face
        the learned step hands to the network (p_TR > 2 min(pL, pR)).  Returns
        the rows (at most capacity) and, with strong=True, the number of such
        faces as a third value.  check=False: the physics status bits of the
        step (non-physical values, which the reference only warns about) do
        not raise; argument, CUDA and capacity errors still do."""
        x = np.zeros((capacity, 4), dtype=np.float32)
        t = np.zeros(capacity, dtype=np.float32)
        cnt = ctypes.c_longlong()
        if strong:
            st = self.L.mlh_pstar_harvest_strong(self.h, _fptr(x), _fptr(t), capacity, ctypes.byref(cnt))
        else:
            st = self.L.mlh_pstar_harvest(self.h, stride, _fptr(x), _fptr(t), capacity, ctypes.byref(cnt))
        hard = (1 << 20) | (1 << 21) | (1 << 22) | (1 << 23) | (1 << 11)
        if st != 0 and (check or (st & hard)):
            raise MLHError(st, "mlh_pstar_harvest", self.L.mlh_last_error().decode())
        k = min(cnt.value, capacity)
        if strong:
            return x[:k], t[:k], cnt.value
        return x[:k], t[:k]

    def smoothing_lengths(self, n_ngb: float):
        """Per-particle smoothing lengths of the current state (mlh_smoothing_lengths):
        (h, effective neighbour number, number of particles clamped at kernel_size)."""
        h = np.empty(self.host.n)
        ne = np.empty(self.host.n)
        cl = ctypes.c_longlong()
        dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        st = self.L.mlh_smoothing_lengths(self.h, float(n_ngb), dp(h), dp(ne), ctypes.byref(cl))
        if st != 0:
            raise MLHError(st, "mlh_smoothing_lengths", self.L.mlh_last_error().decode())
        return h, ne, int(cl.value)

    def prepare(self, dt_max: float = 0.0):
        """Density, dt and limited gradients of the current state (mlh_prepare)."""
        st = self.L.mlh_prepare(self.h, dt_max)
        if st != 0:
            raise MLHError(st, "mlh_prepare", self.L.mlh_last_error().decode())

    def autotune(self, trial_steps: int = 1) -> dict:
        t = Tuning()
        st = self.L.mlh_autotune(self.h, trial_steps, ctypes.byref(t))
        if st != 0:
            raise MLHError(st, "mlh_autotune", self.L.mlh_last_error().decode())
        return {k: getattr(t, k) for k, _ in Tuning._fields_}

    def set_tuning(self, tuning: dict):
        """Launch shapes (mlh_set_tuning); face_split, link_overlap and
        learned_guess default to 1, persistent_binning to 0, fp32_filters to
        3 (both)."""
        dflt = {"face_split": 1, "link_overlap": 1, "persistent_binning": 0, "fp32_filters": 3, "learned_guess": 1}
        t = Tuning(**{k: int(tuning.get(k, dflt[k]) if k in dflt else tuning[k]) for k, _ in Tuning._fields_})
        st = self.L.mlh_set_tuning(self.h, ctypes.byref(t))
        if st != 0:
            raise MLHError(st, "mlh_set_tuning", self.L.mlh_last_error().decode())

    def step(self, nsteps: int = 1, dt_max: float = 0.0, check: bool = True) -> StepStats:
        stats = StepStats()
        st = self.L.mlh_step(self.h, nsteps, dt_max, ctypes.byref(stats))
        if check and st != 0:
            raise MLHError(st, "mlh_step", self.L.mlh_last_error().decode())
        return stats

    def get_state(self) -> dict:
        st = self.L.mlh_get_fields(self.h, ctypes.byref(self.host.view))
        if st != 0:
            raise MLHError(st, "mlh_get_fields", self.L.mlh_last_error().decode())
        keys = ("x", "y", "vx", "vy", "m", "u") + (("z", "vz") if self.dim == 3 else ())
        return {k: self.host.arrays[k].copy() for k in keys}

    def set_state(self, pset):
        """Replace the state (mlh_set_fields); a particle count other than the
        context's raises and leaves the context and its host buffers as they
        were."""
        host = HostState(pset)
        st = self.L.mlh_set_fields(self.h, ctypes.byref(host.view))
        if st != 0:
            raise MLHError(st, "mlh_set_fields", self.L.mlh_last_error().decode())
        self.host = host

    def get(self, name: str) -> np.ndarray:
        cnt = ctypes.c_longlong()
        st = self.L.mlh_stage_array(self.h, name.encode(), None, 0, ctypes.byref(cnt))
        if st != 0:
            raise MLHError(st, f"mlh_stage_array({name})", self.L.mlh_last_error().decode())
        dt = np.uint32 if name in ("nnl",) else (np.int32 if name in INT_ARRAYS else np.float64)
        out = np.empty(cnt.value, dtype=dt)
        st = self.L.mlh_stage_array(self.h, name.encode(), out.ctypes.data_as(ctypes.c_void_p), cnt.value,
                                    ctypes.byref(cnt))
        if st != 0:
            raise MLHError(st, f"mlh_stage_array({name})", self.L.mlh_last_error().decode())
        return out

    def set_kernel_timing(self, on: bool):
        self.L.mlh_set_kernel_timing(self.h, 1 if on else 0)

    def reset_kernel_times(self):
        self.L.mlh_reset_kernel_times(self.h)

    def kernel_times(self) -> dict:
        k = 16
        names = (ctypes.c_char_p * k)()
        launches = (ctypes.c_longlong * k)()
        ms = (ctypes.c_double * k)()
        cnt = self.L.mlh_kernel_times(self.h, names, launches, ms, k)
        return {names[i].decode(): (int(launches[i]), float(ms[i])) for i in range(cnt)}

    def close(self):
        if getattr(self, "h", None):
            self.L.mlh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
