"""Run-time form of the reference's configuration.

The reference splits its settings between config.info (read by
demonstrator/src/main.cpp:55-85: timeStep, timeEnd, h5DumpInterval,
periodicBoxLimits, kernelSize, gamma) and compile-time macros in
demonstrator/include/parameter.h:9-74 (DIM, PERIODIC_BOUNDARIES,
ADAPTIVE_TIMESTEP, CFL, SLOPE_LIMITING, BETA, PAIRWISE_LIMITER, PSI_1, PSI_2,
MESHLESS_FINITE_MASS, MOVE_PARTICLES, FIRST_ORDER_QUAD_POINT).  Here all of them
are fields of one record, mirrored field for field by `mlh_config` in
include/mlh.h.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, fields, replace


@dataclass
class MFVConfig:
    dim: int = 2
    periodic: bool = True
    adaptive_timestep: bool = True
    slope_limiting: bool = True
    pairwise_limiter: bool = False
    meshless_finite_mass: bool = False
    move_particles: bool = True
    first_order_quad_point: bool = True
    # abs() binding of the reference's limiters: False = fabs, True = the
    # int abs(int) binding a build without <math.h>/<stdlib.h> gets
    int_abs: bool = False
    # apply the pairwise limiter on periodic-image faces (the reference's
    # ghost path, Particles.cpp:2533-2683, does not)
    image_pairwise_limiter: bool = False
    riemann_max_iter: int = 100
    max_neighbours: int = 0  # 0: chosen from the dimension
    box_lo: tuple = (0.0, 0.0, 0.0)
    box_hi: tuple = (1.0, 1.0, 0.0)
    kernel_size: float = 0.025231
    gamma: float = 5.0 / 3.0
    cfl: float = 0.3
    time_step: float = 0.005
    beta: float = 4.0
    psi1: float = 0.5
    psi2: float = 0.25
    riemann_tol: float = 1e-10
    # per-particle smoothing lengths (no reference counterpart): each step
    # solves h_i <= kernel_size so that the effective neighbour number is n_ngb
    n_ngb: float = 0.0
    adaptive_h: bool = False

    @classmethod
    def kelvin_helmholtz(cls, pset, **kw) -> "MFVConfig":
        """testcases/kelvin-helmholtz/parameter.h with ADAPTIVE_TIMESTEP and CFL 0.3."""
        c = cls(dim=2, periodic=True, cfl=0.3, beta=4.0, pairwise_limiter=False,
                box_lo=tuple(pset.box_lo), box_hi=tuple(pset.box_hi),
                kernel_size=pset.kernel_size, gamma=pset.gamma)
        return replace(c, **kw)

    @classmethod
    def sedov(cls, pset, periodic: bool = True, **kw) -> "MFVConfig":
        """testcases/sedov/parameter.h: CFL 0.25, BETA 1, PAIRWISE_LIMITER 1."""
        c = cls(dim=3, periodic=periodic, cfl=0.25, beta=1.0, pairwise_limiter=True,
                box_lo=tuple(pset.box_lo), box_hi=tuple(pset.box_hi),
                kernel_size=pset.kernel_size, gamma=pset.gamma)
        return replace(c, **kw)


_INT_FIELDS = ["dim", "periodic", "adaptive_timestep", "slope_limiting", "pairwise_limiter",
               "meshless_finite_mass", "move_particles", "first_order_quad_point", "int_abs",
               "image_pairwise_limiter", "riemann_max_iter", "max_neighbours"]
_DBL_FIELDS = ["kernel_size", "gamma", "cfl", "time_step", "beta", "psi1", "psi2", "riemann_tol"]


class CConfig(ctypes.Structure):
    """ctypes image of `mlh_config` (include/mlh.h)."""
    _fields_ = ([(f, ctypes.c_int) for f in _INT_FIELDS]
                + [("box_lo", ctypes.c_double * 3), ("box_hi", ctypes.c_double * 3)]
                + [(f, ctypes.c_double) for f in _DBL_FIELDS]
                + [("n_ngb", ctypes.c_double), ("adaptive_h", ctypes.c_int)])


def to_struct(cfg: MFVConfig, struct_type=CConfig):
    s = struct_type()
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


__all__ = ["MFVConfig", "CConfig", "to_struct", "fields"]
