"""ctypes binding of the host-side I/O of include/mlh_io.h (libmlh.so):
config.info, parameter.h and the reference's HDF5 initial-condition and
snapshot files.  None of it needs a GPU.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import runtime
from .config import CConfig

EXPORTS = ["mlh_default_run_config", "mlh_read_parameter_header", "mlh_read_config_info", "mlh_info_get",
           "mlh_h5_dataset_info", "mlh_h5_read_f64", "mlh_h5_read_i32", "mlh_h5_create", "mlh_h5_add_f64",
           "mlh_h5_add_i32", "mlh_h5_close", "mlh_read_initial_count", "mlh_read_initial_distribution",
           "mlh_write_snapshot"]


class RunConfig(ctypes.Structure):
    """mlh_run_config."""
    _fields_ = [("cfg", CConfig), ("init_file", ctypes.c_char * 1024), ("out_dir", ctypes.c_char * 1024),
                ("time_end", ctypes.c_double), ("h5_dump_interval", ctypes.c_int), ("debug_lvl", ctypes.c_int)]


_declared = False


def lib():
    global _declared
    L = runtime.load()
    if _declared:
        return L
    vp, cp, ip, dp = ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_void_p
    llp = ctypes.POINTER(ctypes.c_longlong)
    L.mlh_default_run_config.argtypes = [ctypes.POINTER(RunConfig)]
    L.mlh_default_run_config.restype = None
    L.mlh_read_parameter_header.argtypes = [cp, ctypes.POINTER(RunConfig)]
    L.mlh_read_config_info.argtypes = [cp, ctypes.POINTER(RunConfig)]
    L.mlh_info_get.argtypes = [cp, cp, ctypes.c_char_p, ip]
    L.mlh_h5_dataset_info.argtypes = [cp, cp, ctypes.POINTER(ctypes.c_int), llp, ctypes.POINTER(ctypes.c_int),
                                      ctypes.POINTER(ctypes.c_int)]
    L.mlh_h5_read_f64.argtypes = [cp, cp, dp, ctypes.c_longlong]
    L.mlh_h5_read_i32.argtypes = [cp, cp, dp, ctypes.c_longlong]
    L.mlh_h5_create.argtypes = [cp, ctypes.POINTER(vp)]
    L.mlh_h5_add_f64.argtypes = [vp, cp, ip, llp, dp]
    L.mlh_h5_add_i32.argtypes = [vp, cp, ip, llp, dp]
    L.mlh_h5_close.argtypes = [vp]
    L.mlh_read_initial_count.argtypes = [cp, ctypes.POINTER(ctypes.c_int)]
    L.mlh_read_initial_distribution.argtypes = [cp, ip, ctypes.POINTER(runtime.ParticlesView), dp]
    L.mlh_write_snapshot.argtypes = [cp, ip, ctypes.POINTER(runtime.ParticlesView), dp, dp, dp, dp, dp,
                                     ctypes.c_double]
    for f in EXPORTS[1:]:
        getattr(L, f).restype = ctypes.c_int
    _declared = True
    return L


def _check(st, where):
    if st != 0:
        raise runtime.MLHError(st, where, runtime.load().mlh_last_error().decode())


def default_run_config() -> RunConfig:
    r = RunConfig()
    lib().mlh_default_run_config(ctypes.byref(r))
    return r


def read_run_config(config_info: str, parameter_h: str | None = None) -> RunConfig:
    """parameter.h switches (when given) then config.info, as the `mlh` driver reads them."""
    L = lib()
    r = default_run_config()
    if parameter_h:
        _check(L.mlh_read_parameter_header(parameter_h.encode(), ctypes.byref(r)), "parameter.h")
    _check(L.mlh_read_config_info(config_info.encode(), ctypes.byref(r)), "config.info")
    return r


def read_parameter_header(path: str) -> RunConfig:
    r = default_run_config()
    _check(lib().mlh_read_parameter_header(path.encode(), ctypes.byref(r)), "parameter.h")
    return r


def info_get(path: str, key: str) -> str:
    buf = ctypes.create_string_buffer(4096)
    _check(lib().mlh_info_get(path.encode(), key.encode(), buf, len(buf)), "mlh_info_get")
    return buf.value.decode()


def h5_info(path: str, name: str):
    """(rank, shape, 'f'|'i', element size) of a dataset."""
    rank, cls, size = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    dims = (ctypes.c_longlong * 2)()
    _check(lib().mlh_h5_dataset_info(path.encode(), name.encode(), ctypes.byref(rank), dims, ctypes.byref(cls),
                                     ctypes.byref(size)), "mlh_h5_dataset_info")
    shape = (dims[0],) if rank.value == 1 else (dims[0], dims[1])
    return rank.value, shape, "f" if cls.value == 0 else "i", size.value


def h5_read(path: str, name: str) -> np.ndarray:
    """A dataset as float64 (floating-point data) or int32 (integers)."""
    _, shape, kind, _ = h5_info(path, name)
    out = np.empty(shape, dtype=np.float64 if kind == "f" else np.int32)
    fn = lib().mlh_h5_read_f64 if kind == "f" else lib().mlh_h5_read_i32
    _check(fn(path.encode(), name.encode(), out.ctypes.data, out.size), "mlh_h5_read")
    return out


def h5_write(path: str, datasets: dict):
    """Writes {name: array} (float arrays as float64, integer arrays as int32)."""
    L = lib()
    w = ctypes.c_void_p()
    _check(L.mlh_h5_create(path.encode(), ctypes.byref(w)), "mlh_h5_create")
    try:
        for name, a in datasets.items():
            a = np.asarray(a)
            isf = a.dtype.kind == "f"
            a = np.ascontiguousarray(a, dtype=np.float64 if isf else np.int32)
            dims = (ctypes.c_longlong * 2)(*(list(a.shape) + [1])[:2])
            fn = L.mlh_h5_add_f64 if isf else L.mlh_h5_add_i32
            _check(fn(w, name.encode(), a.ndim, dims, a.ctypes.data), "mlh_h5_add")
    except Exception:
        L.mlh_h5_close(w)
        raise
    _check(L.mlh_h5_close(w), "mlh_h5_close")


def write_initial_distribution(path: str, pset, material_id=None):
    """An initial-condition file as the reference's generators write it:
    /x, /v (N x DIM), /m, /u, /materialId."""
    d = pset.dim
    X = np.stack([pset.x, pset.y, pset.z][:d], axis=1)
    V = np.stack([pset.vx, pset.vy, pset.vz][:d], axis=1)
    mat = np.zeros(pset.n, dtype=np.int32) if material_id is None else np.asarray(material_id, dtype=np.int32)
    h5_write(path, {"x": X, "v": V, "m": pset.m, "u": pset.u, "materialId": mat})


def read_initial_distribution(path: str, dim: int):
    """(state dict x, y, (z), vx, vy, (vz), m, u; materialId) of an initial-condition file."""
    L = lib()
    n = ctypes.c_int()
    _check(L.mlh_read_initial_count(path.encode(), ctypes.byref(n)), "mlh_read_initial_count")
    hs = runtime.HostState(n=n.value, dim=dim)
    mat = np.zeros(n.value, dtype=np.int32)
    _check(L.mlh_read_initial_distribution(path.encode(), dim, ctypes.byref(hs.view), mat.ctypes.data),
           "mlh_read_initial_distribution")
    keys = ["x", "y", "vx", "vy", "m", "u"] + (["z", "vz"] if dim == 3 else [])
    return {k: hs.arrays[k].copy() for k in keys}, mat
