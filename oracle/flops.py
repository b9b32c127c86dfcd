"""TEST INFRASTRUCTURE (oracle): algorithmic operation counts of the MFV step.

The operation-counting build of the oracle (liborc_count.so: the oracle
computing in a double that counts the operations done on it, flop_count.hpp)
runs whole steps of a workload; its per-stage counts, divided by the units
each stage works on, are the algorithmic operations per unit of the
reference's method, independent of how the GPU kernels implement it.

Every operation weighs 1 (an addition, subtraction, multiplication,
division, square root or pow call), an explicit fused multiply-add 2.
Comparisons, negation, fabs and arithmetic on configuration constants are
not counted.

The stages of the reference that each kernel of the GPU step performs, and
the unit it is counted per:

  neighbours_density  nns + density + pressure (ORC_STAGE_NNS..PRESSURE)  particle
  timestep            compGlobalTimestep                                   particle
  gradients_limiter   compPsijTilde + gradient + slopeLimiter              particle
  faces_riemann       compEffectiveFace + compRiemannStatesLR +            canonical face
                      solveRiemannProblems
  gather_update       collectFluxes + updateStateAndPosition               particle
  smoothing_lengths   per-particle h solve (adaptive h only)               particle

The reference computes the effective face and the states on every slot of a
face (a slot's states are those of both sides) and solves each face from one
of its two slots (Particles.cpp:1787-1911, ENFORCE_FLUX_SYM): faces_riemann
counts one slot's share of the first two stages, (face + states) / slots per
face, and the Riemann solves of the canonical faces.

    python oracle/flops.py --workload sedov --n-side 32 --steps 3
"""
from __future__ import annotations

import argparse
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import oracle  # noqa: E402

KERNELS = {
    "neighbours_density": (["nns", "density", "pressure"], "particle"),
    "timestep": (["timestep"], "particle"),
    "gradients_limiter": (["psi", "gradients", "limiter"], "particle"),
    "faces_riemann": (["riemann"], "face"),
    "gather_update": (["collect", "update"], "particle"),
    "smoothing_lengths": (["hsolve"], "particle"),
}


def flops_of(c: dict) -> int:
    """Operations of one stage's counts: each weighs 1, an FMA 2."""
    return c["add"] + c["mul"] + c["div"] + c["sqrt"] + c["pow"] + 2 * c["fma"]


def count(cfg, pset, steps: int) -> dict:
    """Run `steps` steps in the counting build and return the algorithmic
    operations per unit of each kernel, the totals per particle-step and
    the units seen."""
    o = oracle.Oracle(cfg, pset, counting=True)
    faces = slots = 0
    newton = 0
    for _ in range(steps):
        st = o.step()
        if st & ~((1 << 6) | (1 << 1)):   # anything but vacuum / negative-pressure warnings
            raise RuntimeError(f"oracle step status {st:#x}")
        stats = o.get("stats")
        faces += int(stats[0])
        newton += int(stats[1])
        slots += int(o.get("off")[-1])
    fc = o.flop_counts()
    o.close()
    n_steps_particles = pset.n * steps
    out = {"steps": steps, "particles": pset.n, "faces_per_step": faces / steps,
           "slots_per_step": slots / steps, "newton_iterations_per_face": newton / max(faces, 1),
           "per_unit": {}, "ops_per_unit": {}}
    for k, (stages, unit) in KERNELS.items():
        tot = {op: sum(fc[s][op] for s in stages) for op in oracle.OPS}
        if k == "faces_riemann":
            share = {op: (fc["face"][op] + fc["states"][op]) * faces / max(slots, 1) for op in oracle.OPS}
            tot = {op: tot[op] + share[op] for op in oracle.OPS}
        units = faces if unit == "face" else n_steps_particles
        out["per_unit"][k] = flops_of(tot) / max(units, 1)
        out["ops_per_unit"][k] = {op: tot[op] / max(units, 1) for op in oracle.OPS}
    out["units"] = {k: u for k, (_, u) in KERNELS.items()}
    out["step_per_particle"] = sum(flops_of(fc[s]) for s in oracle.STAGES) / n_steps_particles
    out["stages_per_particle"] = {s: flops_of(fc[s]) / n_steps_particles for s in oracle.STAGES}
    return out


def workload(name: str, n_side: int, seed: int):
    from meshlesshydro_gb300 import ic
    from meshlesshydro_gb300.config import MFVConfig
    if name == "sedov":
        p = ic.sedov(n_side=n_side, seed=seed)
        return MFVConfig.sedov(p, periodic=True), p
    if name == "kh":
        p = ic.kelvin_helmholtz(n_side=n_side, seed=seed)
        return MFVConfig.kelvin_helmholtz(p), p
    raise ValueError(name)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--workload", choices=["sedov", "kh"], default="sedov")
    ap.add_argument("--n-side", type=int, default=32)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--steps", type=int, default=3)
    a = ap.parse_args(argv)
    cfg, p = workload(a.workload, a.n_side, a.seed)
    res = count(cfg, p, a.steps)
    res["workload"] = f"{a.workload} n_side={a.n_side} seed={a.seed}"
    print(json.dumps(res, indent=1))


if __name__ == "__main__":
    main()
