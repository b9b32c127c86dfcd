"""Seeded initial conditions for the MFV step (host side, numpy).

The reference ships no initial-condition files; its generators are
testcases/kelvin-helmholtz/generateIC.py (2D Kelvin-Helmholtz, mass m = rho/N at
:109-111) and testcases/sedov/initial_sedov.py (3D Sedov, needs `seagen`).  These
functions build the same physical set-ups on jittered lattices with a recorded
seed, in the reference's input layout (/x /v /m /u /materialId of
demonstrator/src/InitialDistribution.cpp:11-29), as structure-of-arrays float64.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

GAMMA = 5.0 / 3.0

# kernelSize / lattice spacing for ~20 neighbours in 2D (the 100x100 set-up
# uses h = 0.025231) and for a mean of 32 neighbours on the jittered 3D lattice
# (found by `mean_neighbours` bisection on the seeded 64^3 lattice).
KH_H_OVER_DX = 2.5231
SEDOV_H_OVER_DX = 2.102


@dataclass
class ParticleSet:
    """SoA particle state, the fields of the reference's Particles class."""
    dim: int
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    vx: np.ndarray
    vy: np.ndarray
    vz: np.ndarray
    m: np.ndarray
    u: np.ndarray
    kernel_size: float
    box_lo: tuple = (0.0, 0.0, 0.0)
    box_hi: tuple = (1.0, 1.0, 0.0)
    gamma: float = GAMMA
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.x.shape[0])

    def arrays(self):
        return [self.x, self.y, self.z, self.vx, self.vy, self.vz, self.m, self.u]

    def copy(self) -> "ParticleSet":
        return ParticleSet(self.dim, *(a.copy() for a in self.arrays()), self.kernel_size,
                           self.box_lo, self.box_hi, self.gamma, dict(self.meta))


def cubic_spline(r: np.ndarray, h: float, dim: int) -> np.ndarray:
    """Kernel::cubicSpline (demonstrator/src/Particles.cpp:7-24): support h."""
    h2 = h / 2.0
    sigma = 10.0 / (7.0 * math.pi * h2 * h2) if dim == 2 else 1.0 / (math.pi * h2 * h2 * h2)
    q = r / h2
    w = np.where(q <= 1.0, sigma * (1.0 - 1.5 * q * q * (1.0 - q / 2.0)),
                 np.where(q < 2.0, sigma / 4.0 * (2.0 - q) ** 3, 0.0))
    return w


def kelvin_helmholtz(n_side: int = 100, seed: int = 1, jitter: float = 0.1, delta: float = 0.025,
                     pressure: float = 2.5, amplitude: float = 0.01, gamma: float = GAMMA,
                     kernel_size: float | None = None) -> ParticleSet:
    """2D Kelvin-Helmholtz in the periodic unit square.

    n_side^2 particles on a cell-centred lattice with uniform jitter of
    +-`jitter` lattice spacings per axis; rho = 1 outside and 2 for
    0.25 < y < 0.75 with tanh interfaces of width `delta`; vx = -0.5 / +0.5 with
    the same smoothing; vy = amplitude * sin(4 pi x); uniform pressure.
    """
    rng = np.random.default_rng(seed)
    dx = 1.0 / n_side
    i = np.arange(n_side)
    gx, gy = np.meshgrid(i, i, indexing="xy")  # x fastest
    x = (gx.ravel() + 0.5) * dx + rng.uniform(-jitter, jitter, n_side * n_side) * dx
    y = (gy.ravel() + 0.5) * dx + rng.uniform(-jitter, jitter, n_side * n_side) * dx
    s = 0.5 * (np.tanh((y - 0.25) / delta) - np.tanh((y - 0.75) / delta))
    rho = 1.0 + s
    vx = -0.5 + s
    vy = amplitude * np.sin(4.0 * math.pi * x)
    n = x.shape[0]
    u = pressure / ((gamma - 1.0) * rho)
    m = rho / n
    h = kernel_size if kernel_size is not None else KH_H_OVER_DX * dx
    zeros = np.zeros(n)
    return ParticleSet(2, x, y, zeros.copy(), vx, vy, zeros.copy(), m, u, float(h),
                       (0.0, 0.0, 0.0), (1.0, 1.0, 0.0), gamma,
                       {"setup": "kelvin-helmholtz", "n_side": n_side, "seed": seed, "jitter": jitter,
                        "delta": delta, "amplitude": amplitude})


def lattice_3d(n_side: int, seed: int, jitter: float, lo: float = -0.5, hi: float = 0.5):
    rng = np.random.default_rng(seed)
    dx = (hi - lo) / n_side
    i = np.arange(n_side)
    gz, gy, gx = np.meshgrid(i, i, i, indexing="ij")  # x fastest
    n = n_side ** 3
    x = lo + (gx.ravel() + 0.5) * dx + rng.uniform(-jitter, jitter, n) * dx
    y = lo + (gy.ravel() + 0.5) * dx + rng.uniform(-jitter, jitter, n) * dx
    z = lo + (gz.ravel() + 0.5) * dx + rng.uniform(-jitter, jitter, n) * dx
    return x, y, z, dx


def mean_neighbours(x, y, z, h: float, box: float | None = 1.0) -> float:
    """Mean number of neighbours j != i with |x_j - x_i| < h (periodic box)."""
    from scipy.spatial import cKDTree
    pts = np.stack([x, y, z], axis=1)
    if box is not None:
        pts = np.mod(pts + 0.5 * box, box)
    tree = cKDTree(pts, boxsize=box)
    pairs = tree.count_neighbors(tree, np.nextafter(h, 0.0))
    return (pairs - len(x)) / len(x)


def bisect_kernel_size(x, y, z, dx: float, target: float = 32.0, iters: int = 30) -> float:
    lo, hi = 1.5 * dx, 3.0 * dx
    for _ in range(iters):
        mid = 0.5 * (lo + hi)
        if mean_neighbours(x, y, z, mid) < target:
            lo = mid
        else:
            hi = mid
    return hi


def sedov(n_side: int = 64, seed: int = 2, jitter: float = 0.05, energy: float = 1.0,
          p_background: float = 1e-5, gamma: float = GAMMA, periodic: bool = True,
          kernel_size: float | None = None) -> ParticleSet:
    """3D Sedov blast in the cube [-0.5, 0.5]^3.

    n_side^3 particles on a cell-centred lattice with +-`jitter` spacings of
    uniform jitter; rho = 1, v = 0, P = p_background; `energy` deposited as
    specific internal energy weighted by the cubic spline of support h around
    the origin: u_i += E W(r_i, h) / sum_j m_j W(r_j, h) (so sum m_i du_i = E).
    """
    x, y, z, dx = lattice_3d(n_side, seed, jitter)
    n = x.shape[0]
    h = kernel_size if kernel_size is not None else SEDOV_H_OVER_DX * dx
    m = np.full(n, 1.0 / n)
    u = np.full(n, p_background / ((gamma - 1.0) * 1.0))
    r = np.sqrt(x * x + y * y + z * z)
    w = cubic_spline(r, h, 3)
    u = u + energy * w / np.sum(m * w)
    zeros = np.zeros(n)
    return ParticleSet(3, x, y, z, zeros.copy(), zeros.copy(), zeros.copy(), m, u, float(h),
                       (-0.5, -0.5, -0.5), (0.5, 0.5, 0.5), gamma,
                       {"setup": "sedov", "n_side": n_side, "seed": seed, "jitter": jitter,
                        "energy": energy, "p_background": p_background, "periodic": periodic})


def multi_blast(n_side: int = 32, n_blasts: int = 16, seed: int = 11, jitter: float = 0.05,
                energy: float = 0.1, p_background: float = 1e-2, gamma: float = GAMMA) -> ParticleSet:
    """Many Sedov blasts in one periodic cube [-0.5, 0.5]^3: the Sedov lattice
    and background of `sedov`, with energy/n_blasts deposited around each of
    n_blasts centres drawn uniformly in the cube (seeded), kernel-weighted
    over periodic distances as `sedov` deposits its one blast.  A workload
    full of strong shocks across the faces of every blast's rim, where the
    two-rarefaction guess of the Riemann solver is poor (about 5 % of the
    faces need 4 or more Newton steps from it with the default energy and
    background, which keep every step free of vacuum and negative pressures);
    no counterpart in the reference's test cases."""
    x, y, z, dx = lattice_3d(n_side, seed, jitter)
    n = x.shape[0]
    h = SEDOV_H_OVER_DX * dx
    m = np.full(n, 1.0 / n)
    u = np.full(n, p_background / ((gamma - 1.0) * 1.0))
    rng = np.random.default_rng(seed + 7919)
    centres = rng.uniform(-0.5, 0.5, (n_blasts, 3))
    for c in centres:
        d = [np.remainder(a - ca + 0.5, 1.0) - 0.5 for a, ca in zip((x, y, z), c)]
        w = cubic_spline(np.sqrt(d[0] ** 2 + d[1] ** 2 + d[2] ** 2), h, 3)
        u = u + (energy / n_blasts) * w / np.sum(m * w)
    zeros = np.zeros(n)
    return ParticleSet(3, x, y, z, zeros.copy(), zeros.copy(), zeros.copy(), m, u, float(h),
                       (-0.5, -0.5, -0.5), (0.5, 0.5, 0.5), gamma,
                       {"setup": "multi_blast", "n_side": n_side, "n_blasts": n_blasts, "seed": seed,
                        "jitter": jitter, "energy": energy, "p_background": p_background})


def concatenate(members) -> ParticleSet:
    """The particle sets of an ensemble stored back to back (member order)."""
    first = members[0]
    cat = [np.concatenate([getattr(m, k) for m in members]) for k in ("x", "y", "z", "vx", "vy", "vz", "m", "u")]
    return ParticleSet(first.dim, *cat, first.kernel_size, first.box_lo, first.box_hi, first.gamma,
                       {"setup": "ensemble", "members": len(members)})


def kh_ensemble(n_members: int = 256, seed: int = 7, n_min: int = 2500, n_max: int = 40000,
                amp_min: float = 0.005, amp_max: float = 0.05):
    """Uneven ensemble of 2D Kelvin-Helmholtz runs: particle counts drawn
    log-uniformly in [n_min, n_max] (lattice side round(sqrt(N)), so N := side^2),
    vy amplitude uniform in [amp_min, amp_max], kernelSize 2.5231 spacings each."""
    rng = np.random.default_rng(seed)
    logn = rng.uniform(math.log(n_min), math.log(n_max), n_members)
    amps = rng.uniform(amp_min, amp_max, n_members)
    out = []
    for k in range(n_members):
        side = int(round(math.sqrt(math.exp(logn[k]))))
        out.append(kelvin_helmholtz(n_side=side, seed=seed * 100003 + k, amplitude=float(amps[k])))
    return out

