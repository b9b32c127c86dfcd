"""The C-ABI library loads and exports every symbol include/mlh.h declares
(no compute calls: this runs without a GPU)."""
import os
import re

from meshlesshydro_gb300 import build, runtime

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions(header="mlh.h"):
    text = open(os.path.join(ROOT, "include", header)).read()
    decl = r"^(?:int|void|double|const char \*)\s*\*?\s*(mlh_[a-z_0-9]+)\s*\("
    return sorted(set(re.findall(decl, text, flags=re.MULTILINE)))


def test_header_and_exports_agree():
    build.build()
    L = runtime.load()
    names = declared_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(runtime.EXPORTS)
    assert L.mlh_abi_version() == 4
    from meshlesshydro_gb300 import io
    io_names = declared_functions("mlh_io.h")
    for n in io_names:
        assert hasattr(L, n), n
    assert set(io_names) == set(io.EXPORTS)


def test_create_without_gpu_fails_cleanly():
    import ctypes
    from meshlesshydro_gb300 import ic
    from meshlesshydro_gb300.config import MFVConfig, to_struct
    L = runtime.load()
    p = ic.kelvin_helmholtz(n_side=8, seed=1)
    hs = runtime.HostState(p)
    cfg = to_struct(MFVConfig.kelvin_helmholtz(p))
    h = ctypes.c_void_p()
    import torch
    st = L.mlh_create(ctypes.byref(cfg), ctypes.byref(hs.view), ctypes.byref(h))
    if not torch.cuda.is_available():
        assert st == (1 << 22)  # MLH_ERR_NO_DEVICE
    else:
        assert st == 0
        L.mlh_destroy(h)
    # invalid arguments are rejected before touching the device
    cfg.dim = 4
    assert L.mlh_create(ctypes.byref(cfg), ctypes.byref(hs.view), ctypes.byref(h)) == (1 << 20)
    # adaptive smoothing lengths need a target above the particle's own count
    cfg.dim = 2
    cfg.adaptive_h = 1
    cfg.n_ngb = 5.0
    assert L.mlh_create(ctypes.byref(cfg), ctypes.byref(hs.view), ctypes.byref(h)) == (1 << 20)
