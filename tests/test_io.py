"""Host-side I/O of the reference's run (include/mlh_io.h, CPU only): the
config.info and parameter.h readers and the HDF5 initial-condition and
snapshot files.  libhdf5 and h5py are absent on both machines, so the HDF5
code is checked against a second, test-only implementation of the file
format (tests/h5spec.py) in both directions."""
import os

import numpy as np
import pytest

import h5spec
from meshlesshydro_gb300 import build, ic, io

REF = __import__("oracle").reference_root()


@pytest.fixture(scope="module", autouse=True)
def _lib():
    build.build()


CONFIG = """; initial distribution
initFile   ics/kh.h5   ; trailing comment
outDir "out dir"

timeStep .002
timeEnd 0.1
h5DumpInterval 5
periodicBoxLimits
{
    lowerX -0.5
    lowerY 0.
    lowerZ 0.
    upperX 0.5
    upperY 1.
    upperZ 0.
}
kernelSize 0.0252
gamma 1.4
"""

PARAMS = """#ifndef DEMONSTRATOR_PARAMETER_H
#define DEMONSTRATOR_PARAMETER_H
#define DIM 2 // two dimensions
#define PERIODIC_BOUNDARIES 1
/* a block
   comment */
#define CFL .25
#define MAX_NUM_INTERACTIONS 300
#define SLOPE_LIMITING 1
#define BETA 2.
#define FIRST_ORDER_QUAD_POINT 1
#define ENFORCE_FLUX_SYM 1
#define DEBUG_LVL 0
#endif
"""


def test_config_and_parameters(tmp_path):
    c = tmp_path / "config.info"
    c.write_text(CONFIG)
    p = tmp_path / "parameter.h"
    p.write_text(PARAMS)
    r = io.read_run_config(str(c), str(p))
    assert r.init_file == b"ics/kh.h5" and r.out_dir == b"out dir"
    assert r.cfg.time_step == 0.002 and r.time_end == 0.1 and r.h5_dump_interval == 5
    assert r.cfg.kernel_size == 0.0252 and r.cfg.gamma == 1.4
    assert list(r.cfg.box_lo)[:2] == [-0.5, 0.0] and list(r.cfg.box_hi)[:2] == [0.5, 1.0]
    # switches the header does not define read as 0, as in #if
    assert (r.cfg.dim, r.cfg.periodic, r.cfg.adaptive_timestep, r.cfg.pairwise_limiter) == (2, 1, 0, 0)
    assert (r.cfg.slope_limiting, r.cfg.first_order_quad_point, r.cfg.move_particles) == (1, 1, 0)
    assert r.cfg.cfl == 0.25 and r.cfg.beta == 2.0 and r.cfg.max_neighbours == 300 and r.debug_lvl == 0
    assert io.info_get(str(c), "periodicBoxLimits.upperY") == "1."
    with pytest.raises(Exception):
        io.info_get(str(c), "periodicBoxLimits.upperW")


@pytest.mark.parametrize("bad", ["#define DIM 4\n", "#define DIM 3\n#define RUNSPH 1\n",
                                 "#define DIM 3\n#define ENFORCE_FLUX_SYM 0\n",
                                 "#define DIM 3\n#define ADAPTIVE_TIMESTEP 1\n",
                                 "#define DIM 3\n#define BETA four\n"])
def test_parameter_header_rejects(tmp_path, bad):
    p = tmp_path / "parameter.h"
    p.write_text(bad)
    with pytest.raises(Exception):
        io.read_parameter_header(str(p))


def test_config_missing_key(tmp_path):
    c = tmp_path / "config.info"
    c.write_text(CONFIG.replace("gamma 1.4\n", ""))
    with pytest.raises(Exception):
        io.read_run_config(str(c))
    c.write_text(CONFIG.replace("}\n", ""))
    with pytest.raises(Exception):
        io.read_run_config(str(c))


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "testcases")), reason="reference tree not present")
def test_reference_inputs():
    """The reference's own test-case inputs, read where they lie."""
    for case in ("kelvin-helmholtz", "sedov", "fluid-block"):
        d = os.path.join(REF, "testcases", case)
        r = io.read_run_config(os.path.join(d, "config.info"), os.path.join(d, "parameter.h"))
        assert r.cfg.kernel_size > 0 and r.cfg.gamma > 1 and r.h5_dump_interval > 0
    kh = io.read_parameter_header(os.path.join(REF, "testcases", "kelvin-helmholtz", "parameter.h"))
    assert (kh.cfg.dim, kh.cfg.periodic, kh.cfg.adaptive_timestep, kh.cfg.pairwise_limiter) == (2, 1, 0, 0)
    assert kh.cfg.max_neighbours == 400 and kh.cfg.beta == 4.0
    sd = io.read_parameter_header(os.path.join(REF, "testcases", "sedov", "parameter.h"))
    assert sd.cfg.dim == 3 and sd.cfg.periodic == 0
    r = io.read_run_config(os.path.join(REF, "demonstrator", "config.info"),
                           os.path.join(REF, "testcases", "kelvin-helmholtz", "parameter.h"))
    assert r.cfg.kernel_size == 0.025 and r.h5_dump_interval == 10


def test_h5_roundtrip_and_independent_reader(tmp_path):
    rng = np.random.default_rng(3)
    data = {"x": rng.normal(size=(37, 3)), "m": rng.uniform(size=37), "noi": rng.integers(-5, 90, 37).astype(np.int32),
            "time": np.array([0.25]), "empty": np.zeros(0)}
    f = str(tmp_path / "a.h5")
    io.h5_write(f, data)
    back = h5spec.read(f)
    assert sorted(back) == sorted(data)
    for k, v in data.items():
        np.testing.assert_array_equal(io.h5_read(f, k), v)
        np.testing.assert_array_equal(back[k], v)
        assert back[k].dtype == (np.float64 if v.dtype.kind == "f" else np.int32)
    assert io.h5_info(f, "/x") == (2, (37, 3), "f", 8)
    with pytest.raises(Exception):
        io.h5_read(f, "nope")


def test_h5_reader_on_other_structures(tmp_path):
    """Files with the structures of other HDF5 writers: superblock v1, a
    two-level group B-tree over several symbol table nodes, continuation
    blocks, NIL and unknown messages, compact storage, big-endian and narrow
    types, version-2 dataspaces."""
    rng = np.random.default_rng(5)
    data = {f"set{k:02d}": rng.normal(size=(11, 2)) for k in range(9)}
    data.update({"f32": rng.normal(size=23).astype(np.float32), "be64": rng.normal(size=7).astype(">f8"),
                 "i64": rng.integers(-2**40, 2**40, 5), "u8": rng.integers(0, 255, 19).astype(np.uint8),
                 "i16be": rng.integers(-300, 300, 4).astype(">i2"), "tiny": np.array([1.5, -2.0])})
    f = str(tmp_path / "b.h5")
    h5spec.write_variant(f, data, leaf_k=2)
    for k, v in data.items():
        out = io.h5_read(f, k)
        if v.dtype.kind == "f":
            np.testing.assert_array_equal(out, v.astype(np.float64))
        elif k == "i64":
            np.testing.assert_array_equal(out, v.astype(np.int32))   # converted as C does (low 32 bits)
        else:
            np.testing.assert_array_equal(out, v.astype(np.int64))


def test_initial_distribution_and_snapshot(tmp_path):
    import ctypes
    from meshlesshydro_gb300 import runtime
    p = ic.sedov(n_side=6, seed=1, energy=0.05)
    f = str(tmp_path / "ic.h5")
    io.write_initial_distribution(f, p, material_id=np.arange(p.n) % 3)
    st, mat = io.read_initial_distribution(f, 3)
    for k in ("x", "y", "z", "vx", "vy", "vz", "m", "u"):
        np.testing.assert_array_equal(st[k], getattr(p, k))
    np.testing.assert_array_equal(mat, np.arange(p.n) % 3)
    # a snapshot (Particles::dump2file layout) reads back as an initial distribution
    hs = runtime.HostState(p)
    rho = np.linspace(1.0, 2.0, p.n)
    P = rho * 0.1
    grad = np.arange(p.n * 3, dtype=np.float64)
    noi = np.full(p.n, 32, dtype=np.int32)
    s = str(tmp_path / "000000.h5")
    dp = lambda a: a.ctypes.data
    L = io.lib()
    assert L.mlh_write_snapshot(s.encode(), 3, ctypes.byref(hs.view), dp(rho), dp(P), dp(grad), dp(noi),
                                dp(mat), 0.125) == 0
    snap = h5spec.read(s)
    assert sorted(snap) == sorted(["time", "totalMass", "energy", "xMomentum", "yMomentum", "zMomentum", "rho",
                                   "m", "u", "P", "noi", "x", "v", "rhoGrad", "materialId"])
    assert snap["time"][0] == 0.125
    M = 0.0
    for v in p.m:
        M += v   # the reference's loop order
    assert snap["totalMass"][0] == M
    np.testing.assert_array_equal(snap["rhoGrad"], grad.reshape(-1, 3))
    np.testing.assert_array_equal(snap["x"][:, 2], p.z)
    st2, mat2 = io.read_initial_distribution(s, 3)
    np.testing.assert_array_equal(st2["u"], p.u)
    np.testing.assert_array_equal(mat2, mat)
