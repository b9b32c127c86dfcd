"""Run a few MFV steps of a seeded set-up on the GPU, for profilers.

    python -m meshlesshydro_gb300.profile_step --setup sedov --n-side 64 --steps 2
    ncu --set full --clock-control none -k regex:k_faces -s 1 -c 1 -o prof \\
        python -m meshlesshydro_gb300.profile_step --setup sedov --n-side 64 --steps 2

--setup ensemble runs the first --members members of the seeded 256-member
Kelvin-Helmholtz ensemble (bench.py's kh_ens256 draws) in one context.
"""
from __future__ import annotations

import argparse

from . import build, ic, runtime
from .config import MFVConfig


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--setup", default="sedov", choices=["sedov", "kh", "ensemble"])
    ap.add_argument("--members", type=int, default=32)
    ap.add_argument("--n-side", type=int, default=64)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--non-periodic", action="store_true")
    a = ap.parse_args(argv)
    build.build()
    if a.setup == "ensemble":
        members = ic.kh_ensemble(n_members=256, seed=7)[:a.members]
        sim = runtime.Simulation(MFVConfig.kelvin_helmholtz(members[0]), members=members)
        n = sim.host.n
    else:
        if a.setup == "sedov":
            p = ic.sedov(n_side=a.n_side, seed=a.seed)
            cfg = MFVConfig.sedov(p, periodic=not a.non_periodic)
        else:
            p = ic.kelvin_helmholtz(n_side=a.n_side, seed=a.seed)
            cfg = MFVConfig.kelvin_helmholtz(p)
        sim = runtime.Simulation(cfg, p)
        n = p.n
    st = sim.step(a.steps)
    print(f"steps {st.steps} particles {n} faces/step {st.faces / max(st.steps, 1):.0f} "
          f"device_ms {st.device_ms:.3f} status {runtime.status_names(st.status)}")


if __name__ == "__main__":
    main()
