"""The C++ host classes with the reference's names (include/mlh.hpp) compile
in a translation unit that defines the reference's parameter.h macros and
take their settings from them; Domain reproduces the reference's grid and
stencil (CPU only: no GPU call is made)."""
import os
import shutil
import subprocess

import pytest

from meshlesshydro_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#define DIM 3
#define PERIODIC_BOUNDARIES 0
#define ADAPTIVE_TIMESTEP 1
#define CFL .25
#define SLOPE_LIMITING 1
#define BETA 1.
#define PAIRWISE_LIMITER 1
#define PSI_1 .5
#define PSI_2 .25
#define MOVE_PARTICLES 1
#define FIRST_ORDER_QUAD_POINT 1
#define MAX_NUM_INTERACTIONS 120
#include "mlh.hpp"
#include <cstdio>
using namespace mlh;
int main() {
    mlh_run_config s = settings_from_macros();
    std::printf("%d %d %d %g %d %g %d %d %d %d %d\n", s.cfg.dim, s.cfg.periodic, s.cfg.adaptive_timestep, s.cfg.cfl,
                s.cfg.slope_limiting, s.cfg.beta, s.cfg.pairwise_limiter, s.cfg.meshless_finite_mass,
                s.cfg.move_particles, s.cfg.first_order_quad_point, s.cfg.max_neighbours);
    Particles p(5);
    for (int i = 0; i < 5; ++i) { p.x[i] = i; p.y[i] = -i; p.z[i] = 2 * i; p.m[i] = 1; p.vx[i] = 1; }
    double lim[6];
    p.getDomainLimits(lim);
    std::printf("%g %g %g %g %g %g %g %g\n", lim[0], lim[1], lim[2], lim[3], lim[4], lim[5], p.sumMass(), p.sumMomentumX());
    double b[6] = {0., 0., 0., 1., 1., 1.};
    Domain d{Domain::Cell(b)};
    d.createGrid(0.3);
    int nc[27];
    d.getNeighborCells(0, nc);
    int outside = 0;
    for (int k = 0; k < 27; ++k) outside += nc[k] < 0;
    std::printf("%d %d %d %d %d %d\n", d.cellsX, d.cellsY, d.cellsZ, d.numGridCells, outside, nc[26]);
    try {
        ConfigParser c("missing.info");
        c.getVal<double>("kernelSize");
    } catch (const Error &e) {
        std::printf("error %d\n", e.status != 0);
    }
    return 0;
}
"""


def test_facade_compiles_and_reads_macros(tmp_path):
    build.build()
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    src = tmp_path / "t.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "t"
    lib_dir = os.path.join(ROOT, "meshlesshydro_gb300")
    subprocess.run([cxx, "-std=c++17", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                    "-L", lib_dir, "-lmlh", "-Wl,-rpath," + lib_dir], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    assert out[0].split() == ["3", "0", "1", "0.25", "1", "1", "1", "0", "1", "1", "120"]
    # getDomainLimits keeps the reference's else-if: a monotone coordinate
    # never updates the minimum after the first element (y decreases)
    lim = [float(v) for v in out[1].split()]
    assert lim[:3] == [0.0, -4.0, 0.0] and lim[3] == 4.0 and lim[5] == 8.0
    assert lim[6] == 5.0 and lim[7] == 5.0
    # floor(1 / 0.3) = 3 cells per axis; cell 0's stencil has 19 cells outside
    assert out[2].split() == ["3", "3", "3", "27", "19", str(1 + 3 + 9)]
    assert out[3] == "error 1"


def test_cli_help():
    build.build()
    exe = os.path.join(ROOT, "meshlesshydro_gb300", "mlh")
    r = subprocess.run([exe, "--help"], capture_output=True, text=True)
    assert r.returncode == 0 and "config.info" in r.stdout
    r = subprocess.run([exe, "-v", "-s"], capture_output=True, text=True)
    assert r.returncode == 2 and "incompatible" in r.stderr
    r = subprocess.run([exe, "-c", "/nonexistent/config.info"], capture_output=True, text=True)
    assert r.returncode == 1 and "cannot open" in r.stderr


C_PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "mlh.h"

int main(void) {
    double x[4] = {0.1, 0.2, 0.3, 0.4}, v[4] = {0., 0., 0., 0.}, m[4] = {1., 1., 1., 1.};
    mlh_config cfg;
    mlh_particles_view view;
    mlh_ctx *ctx = NULL;
    int st;
    memset(&cfg, 0, sizeof cfg);
    memset(&view, 0, sizeof view);
    cfg.dim = 2;
    cfg.periodic = 1;
    cfg.kernel_size = 0.3;
    cfg.gamma = 5. / 3.;
    cfg.box_hi[0] = cfg.box_hi[1] = 1.;
    view.n = 0;                          /* empty: rejected before the device */
    view.x = view.y = x;
    view.vx = view.vy = v;
    view.m = view.u = m;
    st = mlh_create(&cfg, &view, &ctx);
    printf("%d %d %d %s\n", mlh_abi_version(), st == MLH_ERR_INVALID, ctx == NULL, mlh_last_error());
    view.n = 4;
    view.u = NULL;                       /* incomplete view */
    st = mlh_create(&cfg, &view, &ctx);
    printf("%d\n", st == MLH_ERR_INVALID);
    return 0;
}
"""


def test_c99_caller(tmp_path):
    """A plain C99 program against include/mlh.h and libmlh.so (the binding
    an FFI user writes): the ABI version and argument errors, no device."""
    build.build()
    cc = shutil.which("gcc")
    if not cc:
        pytest.skip("no C compiler")
    src = tmp_path / "t.c"
    src.write_text(C_PROGRAM)
    exe = tmp_path / "t"
    lib_dir = os.path.join(ROOT, "meshlesshydro_gb300")
    subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
                    str(src), "-o", str(exe), "-L", lib_dir, "-lmlh", "-Wl,-rpath," + lib_dir], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    assert out[0].startswith("4 1 1 invalid configuration")
    assert out[1] == "1"
