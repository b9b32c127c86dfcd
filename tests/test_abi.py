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


def test_create_rejects_empty_ragged_and_oversized_inputs():
    """Argument checks that run before the device is touched, so the same
    answers come with and without a GPU: an empty particle set, a missing
    coordinate array, a 3D view without z, more particles than the 29-bit
    neighbour index holds, and ensembles whose members are empty, have no
    kernel size or do not add up to the view's particle count."""
    import ctypes
    from meshlesshydro_gb300 import ic
    from meshlesshydro_gb300.config import MFVConfig, to_struct
    INVALID, CAPACITY = 1 << 20, 1 << 23
    L = runtime.load()
    p = ic.kelvin_helmholtz(n_side=8, seed=1)
    cfg = to_struct(MFVConfig.kelvin_helmholtz(p))
    h = ctypes.c_void_p()

    def create(view, c=cfg):
        return L.mlh_create(ctypes.byref(c), ctypes.byref(view), ctypes.byref(h))

    hs = runtime.HostState(p)
    hs.view.n = 0
    assert create(hs.view) == INVALID
    assert b"invalid" in L.mlh_last_error()
    hs = runtime.HostState(p)
    hs.view.x = ctypes.POINTER(ctypes.c_double)()
    assert create(hs.view) == INVALID
    s = ic.sedov(n_side=4, seed=1)
    c3 = to_struct(MFVConfig.sedov(s, periodic=True))
    hs3 = runtime.HostState(s)
    hs3.view.z = ctypes.POINTER(ctypes.c_double)()
    assert create(hs3.view, c3) == INVALID
    # the count alone is checked: no array is read before the rejection
    hs = runtime.HostState(p)
    hs.view.n = (1 << 29)
    assert create(hs.view) == CAPACITY
    assert b"too many particles" in L.mlh_last_error()
    # face ids are 32-bit: particles x neighbour slots / 2 + particles must
    # stay below 2^31 (40 slots in 2D by default: 103 M particles is over)
    hs.view.n = 103_000_000
    assert create(hs.view) == CAPACITY
    assert b"too many faces" in L.mlh_last_error()

    def ensemble(sizes, ks):
        descs = (runtime.MemberDesc * max(len(sizes), 1))()
        for k, (n, hk) in enumerate(zip(sizes, ks)):
            descs[k].n = n
            descs[k].kernel_size = hk
            for a in range(3):
                descs[k].box_lo[a], descs[k].box_hi[a] = 0.0, 1.0
        hs = runtime.HostState(p)
        return L.mlh_ensemble_create(ctypes.byref(cfg), len(sizes), descs, ctypes.byref(hs.view),
                                     ctypes.byref(h))

    n = p.n
    assert ensemble([], []) == INVALID
    assert ensemble([n, 0], [0.1, 0.1]) == INVALID                 # an empty member
    assert ensemble([n // 2, n - n // 2], [0.1, 0.0]) == INVALID   # no kernel size
    assert ensemble([n // 2, n // 2 - 1], [0.1, 0.1]) == INVALID   # one particle left over
    assert b"add up" in L.mlh_last_error()
    assert ensemble([n // 2, n - n // 2 + 1], [0.1, 0.1]) == INVALID


def test_simulation_needs_particles():
    import pytest
    from meshlesshydro_gb300.config import MFVConfig
    from meshlesshydro_gb300 import ic
    p = ic.kelvin_helmholtz(n_side=8, seed=1)
    with pytest.raises(ValueError):
        runtime.Simulation(MFVConfig.kelvin_helmholtz(p))
    with pytest.raises(ValueError):
        runtime.Simulation(MFVConfig.kelvin_helmholtz(p), members=[])
