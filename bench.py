"""Throughput of the GB300 MFV step: particle-updates/s on one GB300.

Default workload: the 3D Sedov blast on a jittered 128^3 lattice (2,097,152
particles) in the periodic cube [-0.5, 0.5]^3, FP64 state, cubic spline with a
mean of 32 neighbours (kernelSize 2.102 lattice spacings), CFL 0.25, BETA 1,
pairwise limiter: the "plain GPU method at scale" configuration.  A step is one
full MFV step (binning, neighbour search, density, dt, gradients, limiter,
faces, exact Riemann solves, flux gather, kick/drift) over all particles.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl mlh|reference]
                    [--workload sedov128|sedov64|kh100|kh_ens256|multi_blast64]
                    [--no-learned] [--no-adaptive] [--no-ensemble] [--no-cpu-baseline]

Prints one JSON line.  Beside the headline it reports, for the default
workload: the learned star-pressure guess (trained on faces harvested from the
64^3 Sedov and 100x100 Kelvin-Helmholtz runs, evaluated on the held-out 128^3
workload and on a many-blast workload full of strong shocks), per-particle
smoothing lengths, and the 256-member Kelvin-Helmholtz ensemble batched
against its members run one after another.  --impl reference times the CPU
restatement of the reference's serial code (the oracle; the reference itself
cannot be built on the GPU host) on every host core, over the workload itself
(a 100x100 KH member-sized set-up for the ensemble), with its serial rate on
a small sample beside.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

WORKLOADS = {
    "sedov128": dict(kind="sedov", n_side=128, periodic=True),
    "sedov64": dict(kind="sedov", n_side=64, periodic=True),
    "kh100": dict(kind="kh", n_side=100),
    # 256 independent 2D KH runs, N log-uniform in [2500, 40000], one context
    "kh_ens256": dict(kind="ensemble", members=256),
    # 64 blasts in the periodic 64^3 cube: strong shocks everywhere (energy
    # 0.02 in all: the blast-to-background pressure ratio of 16 blasts of
    # energy 0.1 in all on 24^3)
    "multi_blast64": dict(kind="multi_blast", n_side=64, n_blasts=64, energy=0.02),
}
METRIC = "particle-updates/s per MFV step on 1 GB300"
# kernels launched by one plain mlh_step iteration (csrc/mlh_kernels.cu,
# launch_step): binning (k_bounds_partial, k_bounds_final, k_assign, 3 scan
# kernels, k_fill_cells, k_sort_cells), k_neighbours, face links (3 scan
# kernels, k_link), k_timestep, k_dt_final, k_gradients, the face pass
# (k_faces_block, or k_faces first pass + second Newton pass), k_update,
# k_advance_time
LAUNCHES_PER_STEP = 20

# What each kernel of the step executes per unit (particle, or canonical
# face for the face pass), from ncu captures of the same kernels: FP64
# operations (2 x DFMA + DADD + DMUL thread instructions per unit) and DRAM
# bytes (read + write per unit); 3D on the 64^3 periodic Sedov step (the time
# step's single-precision bounds inside the gradients' first pass and its FP64
# v_sig for the few candidate particles in k_timestep, the face pass as its
# first pass and the second Newton pass over the queue), 2D on the 256-member
# Kelvin-Helmholtz ensemble (the face pass with the unfinished faces
# continued inside the block).  These are executed, not
# algorithmic, operations: a kernel cannot execute more than the FP64 pipe
# issues, so the rates they give are bounded by the pipe's peak.
KERNEL_UNITS = {"neighbours_density": "particle", "timestep": "particle", "gradients_limiter": "particle",
                "face_links": "particle", "faces_riemann": "face", "gather_update": "particle"}
KERNEL_EXEC = {
    3: {"neighbours_density": (1026.1, 870.9), "timestep": (0.0, 4.1), "gradients_limiter": (2906.7, 1803.9),
        "face_links": (0.0, 1007.7), "faces_riemann": (537.7, 300.9), "gather_update": (212.0, 1534.5)},
    2: {"neighbours_density": (592.7, 887.2), "timestep": (0.0, 8.5), "gradients_limiter": (1126.9, 2074.6),
        "face_links": (0.0, 876.0), "faces_riemann": (344.3, 180.8), "gather_update": (120.0, 975.6)},
}
# FP64 thread instructions (DFMA + DADD + DMUL) per unit of the same
# captures: what the FP64 pipe issues, each instruction one lane-slot
KERNEL_FP64_INSTR = {
    3: {"neighbours_density": 791.1, "timestep": 0.0, "gradients_limiter": 1845.3, "face_links": 0.0,
        "faces_riemann": 353.5, "gather_update": 195.0},
    2: {"neighbours_density": 441.7, "timestep": 0.0, "gradients_limiter": 747.7, "face_links": 0.0,
        "faces_riemann": 244.4, "gather_update": 107.0},
}
# FP64 pipe active (sm__pipe_fp64_cycles_active over elapsed cycles) of the
# same captures
KERNEL_FP64_PIPE = {
    3: {"neighbours_density": 0.588, "timestep": 0.546, "gradients_limiter": 0.840, "faces_riemann": 0.878,
        "gather_update": 0.764, "face_links": 0.0},
    2: {"neighbours_density": 0.716, "timestep": 0.656, "gradients_limiter": 0.766, "faces_riemann": 0.858,
        "gather_update": 0.840, "face_links": 0.0},
}
# Operations of the reference's method per unit, counted by the
# operation-counting build of the oracle (oracle/flops.py; every addition,
# multiplication, division, square root and pow weighs 1, an FMA 2).  This
# counts the reference implementation's work, including rotation matrices,
# repeated kernel evaluations and every candidate of the cell stencil, which
# the kernels here do not execute: it is not a lower bound of the method and
# is reported for comparison only, never as a roofline.
KERNEL_REF_OPS = {
    3: {"neighbours_density": 3618.0, "timestep": 754.0, "gradients_limiter": 7871.0, "face_links": 0.0,
        "faces_riemann": 746.0, "gather_update": 198.0},
    2: {"neighbours_density": 700.0, "timestep": 375.0, "gradients_limiter": 2678.0, "face_links": 0.0,
        "faces_riemann": 339.8, "gather_update": 108.0},
}
FP64_OPS_PER_SM_CYCLE = 4.0   # two fused multiply-adds per SM and cycle


def kernel_rooflines(kernel_ms: dict, dim: int, particles: float, faces: float, fp64_peak_tflops, hbm_peak_gbs):
    """Each kernel of the step against the FP64 and the HBM roofline: its
    time per step (CUDA events), the FP64 operations it executes and the DRAM
    bytes it moves per unit (ncu), the rates they give, and their fractions of
    the measured FP64 FMA peak and HBM copy bandwidth."""
    out = {}
    for k, unit in KERNEL_UNITS.items():
        ms = kernel_ms.get(k)
        if not ms or ms <= 0.0 or dim not in KERNEL_EXEC:
            continue
        fl, by = KERNEL_EXEC[dim][k]
        units = faces if unit == "face" else particles
        s = ms / 1e3
        tf = fl * units / s / 1e12
        gbs = by * units / s / 1e9
        ins = KERNEL_FP64_INSTR.get(dim, {}).get(k)
        ins_rate = ins * units / s if ins is not None else None
        out[k] = {"ms_per_step": ms, "unit": unit, "units_per_step": units,
                  "fp64_flops_per_unit": fl, "fp64_tflops": tf,
                  "fp64_frac": tf / fp64_peak_tflops if fp64_peak_tflops else None,
                  "fp64_instr_per_unit": ins,
                  "fp64_instr_frac": (ins_rate / (fp64_peak_tflops * 1e12 / 2.0))
                  if (ins_rate is not None and fp64_peak_tflops) else None,
                  "fp64_pipe_active_ncu": KERNEL_FP64_PIPE.get(dim, {}).get(k),
                  "dram_bytes_per_unit": by, "hbm_gbs": gbs,
                  "hbm_frac": gbs / hbm_peak_gbs if hbm_peak_gbs else None,
                  "reference_method_ops_per_unit": KERNEL_REF_OPS[dim][k]}
    return out


def step_fp64(dim: int, particles: float, faces: float) -> float:
    """FP64 operations the step's kernels execute per step (ncu per-unit
    figures times the units)."""
    tot = 0.0
    for k, unit in KERNEL_UNITS.items():
        tot += KERNEL_EXEC[dim][k][0] * (faces if unit == "face" else particles)
    return tot


def make_workload(name: str, seed_offset: int = 0):
    from meshlesshydro_gb300 import ic
    from meshlesshydro_gb300.config import MFVConfig
    w = WORKLOADS[name]
    if w["kind"] == "ensemble":
        members = ic.kh_ensemble(n_members=w["members"], seed=7 + seed_offset)
        return members, MFVConfig.kelvin_helmholtz(members[0])
    if w["kind"] == "sedov":
        p = ic.sedov(n_side=w["n_side"], seed=2 + seed_offset)
        return p, MFVConfig.sedov(p, periodic=w["periodic"])
    if w["kind"] == "multi_blast":
        p = ic.multi_blast(n_side=w["n_side"], n_blasts=w["n_blasts"], seed=11 + seed_offset, energy=w["energy"])
        return p, MFVConfig.sedov(p, periodic=True)
    p = ic.kelvin_helmholtz(n_side=w["n_side"], seed=1 + seed_offset)
    return p, MFVConfig.kelvin_helmholtz(p)


def dist_env():
    from meshlesshydro_gb300.replicas import dist_env as env
    return env()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for k, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(k)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name"):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


_T0 = time.perf_counter()


def progress(msg: str):
    """A progress line on stderr (the JSON line alone goes to stdout)."""
    print(f"[bench {time.perf_counter() - _T0:8.1f} s] {msg}", file=sys.stderr, flush=True)


def host_cores():
    return os.cpu_count() or 1


def _oracle_sample(kind: str):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from meshlesshydro_gb300 import ic
    from meshlesshydro_gb300.config import MFVConfig
    oracle.build()
    oracle.set_threads(1)
    if kind == "sedov":
        p = ic.sedov(n_side=32, seed=2)
        return oracle, p, MFVConfig.sedov(p, periodic=True), "32^3 periodic Sedov lattice"
    p = ic.kelvin_helmholtz(n_side=100, seed=1)
    return oracle, p, MFVConfig.kelvin_helmholtz(p), "100x100 Kelvin-Helmholtz set-up"


def _time_oracle(o, seconds_hint, max_steps):
    o.step()  # warm-up
    steps, t0 = 0, time.perf_counter()
    while True:
        o.step()
        steps += 1
        el = time.perf_counter() - t0
        if el >= seconds_hint or steps >= max_steps:
            return steps, el


def _time_oracle_all_threads(oracle, p, cfg, seconds_hint, max_steps):
    """The same restatement with its per-particle loops on every host core
    (OpenMP; the results are the same bits for any thread count): steps per
    second and the thread count.  The reference itself is single-threaded;
    this is reported beside the serial figure, not instead of it."""
    n = oracle.set_threads(0)
    try:
        o = oracle.Oracle(cfg, p)
        steps, el = _time_oracle(o, seconds_hint, max_steps)
    finally:
        oracle.set_threads(1)
    return p.n * steps / el, n


def cpu_baseline_sample(seconds_hint: float = 15.0, kind: str = "sedov"):
    """The oracle (serial CPU restatement of the reference, -O3 as the
    reference's own build) on a bounded sample: whole MFV steps of the 32^3
    Sedov lattice with the workload's particle density and neighbour count
    (the same per-particle work as 128^3), or of the 100x100 Kelvin-Helmholtz
    set-up for the 2D workloads; at the reference's DEBUG_LVL 0 (the value)
    and DEBUG_LVL 1 as its test cases ship it (checkFluxSymmetry every step)."""
    oracle, p, cfg, what = _oracle_sample(kind)
    o = oracle.Oracle(cfg, p)
    steps, el = _time_oracle(o, seconds_hint, 50)
    o1 = oracle.Oracle(cfg, p)
    o1.set_debug_level(1)
    steps1, el1 = _time_oracle(o1, seconds_hint / 3, 20)
    v_all, n_all = _time_oracle_all_threads(oracle, p, cfg, seconds_hint / 3, 50)
    return {"value": p.n * steps / el, "unit": "particle-updates/s", "cores": 1, "kind": "port",
            "host_cores": host_cores(), "host_cpu": cpu_model(),
            "debug_lvl1_value": p.n * steps1 / el1,
            "all_threads_value": v_all, "all_threads": n_all,
            "sample": f"{steps} MFV steps of the {what} ({p.n} particles, the workload's h/dx and neighbour "
                      f"count), serial oracle built -O3 -ffp-contract=off, {el:.1f} s, 1 of {host_cores()} "
                      f"cores of {cpu_model()}; debug_lvl1_value: the same with the reference's DEBUG_LVL 1 "
                      f"flux-symmetry check, {steps1} steps; all_threads_value: the restatement's per-particle "
                      f"loops on {n_all} threads (the reference itself is single-threaded)"}


def run_reference(args):
    """The reference arm: the CPU restatement of the reference's step (the
    reference's own sources are not on the GPU host) on every host core, on
    the workload itself (for the ensemble, on one 100x100 KH member-sized
    set-up), W untimed and K timed steps.  The reference is single-threaded;
    the restatement's per-particle loops run on all cores with the same bits
    (OpenMP), and its serial rate on a small sample is reported beside."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    w = WORKLOADS[args.workload]
    oracle, ps, cfgs, what_s = _oracle_sample("kh" if w["kind"] in ("kh", "ensemble") else "sedov")
    if w["kind"] == "ensemble":
        p, cfg, what = ps, cfgs, what_s + " (one member-sized set-up)"
    else:
        p, cfg = make_workload(args.workload)
        what = f"the {args.workload} workload itself"
    n_threads = oracle.set_threads(0)
    try:
        o = oracle.Oracle(cfg, p)
        for _ in range(args.warmup):
            o.step()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            o.step()
        el = time.perf_counter() - t0
        o.close()
    finally:
        oracle.set_threads(1)
    val = p.n * args.steps / el
    serial_steps, serial_el = _time_oracle(oracle.Oracle(cfgs, ps), 5.0, max(args.steps, 2))
    serial = ps.n * serial_steps / serial_el
    sample = (f"{what} ({p.n} particles), one MFV step per step, CPU restatement of the reference built -O3, "
              f"DEBUG_LVL 0, its per-particle loops on {n_threads} threads (the same bits as serial; the "
              f"reference itself is single-threaded); serial_value: 1 thread on the {what_s} "
              f"({ps.n} particles)")
    line = {"metric": METRIC, "value": val, "unit": "particle-updates/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": args.workload, "sample": sample},
            "cpu_baseline": {"value": val, "unit": "particle-updates/s", "cores": n_threads, "kind": "port",
                             "host_cores": host_cores(), "serial_value": serial,
                             "sample": sample + f", host {cpu_model()}"},
            "e2e": {"value": val, "unit": "particle-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def kernel_breakdown(sim, steps):
    """Per-kernel device times of a few more steps with per-kernel CUDA events
    (which serialise the step's streams), after the timed region."""
    sim.reset_kernel_times()
    sim.set_kernel_timing(True)
    sim.step(max(1, min(steps, 3)))
    sim.set_kernel_timing(False)
    return sim.kernel_times()


def per_step(kt):
    return {k: v[1] / max(v[0], 1) for k, v in kt.items()}


def timed_steps(sim, warmup, steps, check=True):
    """warmup steps, then `steps` timed steps: (stats, wall seconds).
    check=False: non-physical values (which the reference only warns about)
    are reported in the status instead of raised."""
    import torch
    if warmup:
        sim.step(warmup, check=check)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    st = sim.step(steps, check=check)
    torch.cuda.synchronize()
    return st, time.perf_counter() - t0


def train_learned_guess(runtime, budget_rows: int = 10_000_000, epochs: int = 12):
    """The network of the learned star-pressure guess, trained on the GPU
    (mlh_pstar_train) on faces harvested from the plain method's own runs:
    the 64^3 periodic Sedov blast (100 steps: every face the learned step
    hands to the network, at every step, and every 4th face at steps 0, 25,
    50 and 75) and the 100x100 Kelvin-Helmholtz run (100 steps: every face of
    every 5th step), at most budget_rows rows (a seeded subsample beyond).
    A run is harvested up to its first step with non-physical values (which
    the reference only warns about).  The evaluated workloads are other sizes
    and set-ups (the 128^3 Sedov lattice, the 64-blast 64^3 cube)."""
    from meshlesshydro_gb300 import ic
    from meshlesshydro_gb300.config import MFVConfig
    t0 = time.perf_counter()
    xs, ts = [], []
    n_strong = n_sedov = n_kh = 0
    stopped = {}
    p = ic.sedov(n_side=64, seed=2)
    s = runtime.Simulation(MFVConfig.sedov(p, periodic=True), p)
    for k in range(100):
        try:   # a run that reports non-physical values is not harvested further
            if k % 25 == 0:
                x, t = s.harvest(stride=4, capacity=1 << 21)
                n_sedov += x.shape[0]
            else:
                x, t, _ = s.harvest(strong=True, capacity=1 << 20)
                n_strong += x.shape[0]
        except runtime.MLHError as exc:
            stopped["sedov64"] = {"step": k, "status": runtime.status_names(exc.status)}
            break
        xs.append(x); ts.append(t)
    s.close()
    q = ic.kelvin_helmholtz(n_side=100, seed=21)
    s = runtime.Simulation(MFVConfig.kelvin_helmholtz(q), q)
    for k in range(100):
        try:
            if k % 5 == 0:
                x, t = s.harvest(stride=1, capacity=1 << 18)
                xs.append(x); ts.append(t)
                n_kh += x.shape[0]
            else:
                s.step(1)
        except runtime.MLHError as exc:
            stopped["kh100"] = {"step": k, "status": runtime.status_names(exc.status)}
            break
    s.close()
    x = np.concatenate(xs)
    t = np.concatenate(ts)
    rng = np.random.default_rng(0)
    if x.shape[0] > budget_rows:
        keep = rng.choice(x.shape[0], budget_rows, replace=False)
        x, t = x[keep], t[keep]
    t1 = time.perf_counter()
    w, hist = runtime.pstar_train(x, t, epochs=epochs, batch=8192, lr=2e-3, seed=0)
    t2 = time.perf_counter()
    return w, {"rows": int(x.shape[0]), "rows_sedov64_strong": n_strong, "rows_sedov64_every_4th": n_sedov,
               "rows_kh100": n_kh, "harvest_stopped": stopped, "epochs": epochs, "batch": 8192, "lr": 2e-3,
               "loss_first_epoch": float(hist[0]), "loss_last_epoch": float(hist[-1]),
               "harvest_s": t1 - t0, "train_s": t2 - t1}


def network_error(runtime, w, sim_factory):
    """Relative error of the guess p_TR e^y against the converged p* on
    held-out faces: every strong shock and every 64th face of one step of a
    fresh simulation of the evaluated workload."""
    s = sim_factory()
    xs, ts, n = s.harvest(strong=True, capacity=1 << 21, check=False)
    s.close()
    s = sim_factory()
    xa, ta = s.harvest(stride=64, capacity=1 << 21, check=False)
    s.close()
    out = {}
    for name, (x, t) in (("strong", (xs, ts)), ("all_every_64th", (xa, ta))):
        if x.shape[0] == 0:
            out[name] = {"rows": 0}
            continue
        y = runtime.pstar_infer(w, x).astype(np.float64)
        rel = np.abs(np.exp(y - t) - 1.0)
        rel_tr = np.abs(np.exp(-t.astype(np.float64)) - 1.0)   # error of p_TR itself
        out[name] = {"rows": int(x.shape[0]), "median_rel_err": float(np.median(rel)),
                     "p90_rel_err": float(np.quantile(rel, 0.9)),
                     "p_TR_median_rel_err": float(np.median(rel_tr))}
    return out


def learned_vs_plain(runtime, make, w, args, tuning_plain=None, st_plain=None, kt_plain=None, rho_plain=None):
    """The same steps with and without the learned guess, each with the
    autotuner's launch shapes for its own pipeline (so that the learned step
    may take another face-pass structure, and the plain face pipeline where
    the network does not pay: `learned_guess` 0); device time of the timed
    steps.  `learned_over_plain` is the learned context as the autotuner
    configures it; the network pipeline itself (learned_guess 1, the
    autotuner's other shapes) is timed beside it, with its Newton-step
    savings."""
    out = {}
    if st_plain is None:
        sp = make()
        tuning_plain = sp.autotune(2)
        st_plain, _ = timed_steps(sp, args.warmup, args.steps, check=False)
        rho_plain = sp.get("rho")
        kt_plain = kernel_breakdown(sp, args.steps)
        sp.close()
    sl = make()
    sl.set_pstar_weights(w)
    tuning_l = sl.autotune(2)
    st_a, _ = timed_steps(sl, args.warmup, args.steps, check=False)
    sl.close()
    # the network pipeline with the same shapes
    sl = make()
    sl.set_pstar_weights(w)
    sl.set_tuning(dict(tuning_l, learned_guess=1))
    st, _ = timed_steps(sl, args.warmup, args.steps, check=False)
    rho = sl.get("rho")
    kt = kernel_breakdown(sl, args.steps)
    sl.close()
    npart = rho.size
    v_a = npart * st_a.steps / (st_a.device_ms / 1e3)
    v_l = npart * st.steps / (st.device_ms / 1e3)
    v_p = npart * st_plain.steps / (st_plain.device_ms / 1e3)
    saved = st_plain.newton_iterations - st.newton_iterations
    out.update({
        "value": v_a, "plain_value": v_p, "learned_over_plain": v_a / v_p,
        "learned_guess_chosen": int(tuning_l.get("learned_guess", 1)),
        "network_pipeline_value": v_l, "network_pipeline_over_plain": v_l / v_p,
        "newton_iterations_per_face": st.newton_iterations / max(st.faces, 1),
        "plain_newton_iterations_per_face": st_plain.newton_iterations / max(st_plain.faces, 1),
        "iterations_saved": int(saved),
        "iterations_saved_per_learned_face": saved / max(st.learned_faces, 1),
        "learned_faces": int(st.learned_faces), "learned_face_fraction": st.learned_faces / max(st.faces, 1),
        "fallbacks": int(st.newton_fallbacks),
        "fallback_rate": st.newton_fallbacks / max(st.learned_faces, 1),
        "faces_kernel_ms_per_step": per_step(kt).get("faces_riemann"),
        "plain_faces_kernel_ms_per_step": per_step(kt_plain).get("faces_riemann"),
        "density_L1_vs_plain": float(np.sum(np.abs(rho - rho_plain)) / np.sum(np.abs(rho_plain))),
        "tuning": tuning_l, "plain_tuning": tuning_plain,
        "status": runtime.status_names(st.status), "plain_status": runtime.status_names(st_plain.status)})
    return out


def learned_section(runtime, args, make_main, tuning, st_plain, kt_plain, rho_plain):
    """Learned guess: training on the Sedov 64^3 + KH harvest, network error
    on held-out faces, and the learned step against the plain one on the
    bench workload and on the 64-blast 64^3 workload (strong shocks)."""
    progress("learned: harvest and training")
    w, train = train_learned_guess(runtime)
    progress("learned: network error on held-out faces")
    out = {"guess": "p_TR * exp(y) for faces with p_TR > 2 min(pL, pR) where |y| > 0.01, else p_TR; Newton to "
                    "1e-10 relative either way, restarting from p_TR when the network's start does not converge",
           "train": train}
    out["network_error_held_out"] = network_error(runtime, w, make_main)
    progress("learned: main workload")
    out["main_workload"] = learned_vs_plain(runtime, make_main, w, args, tuning, st_plain, kt_plain, rho_plain)
    progress("learned: multi-blast workload")
    pm, cm = make_workload("multi_blast64")
    mk = lambda: runtime.Simulation(cm, pm)
    out["multi_blast64"] = learned_vs_plain(runtime, mk, w, args)
    out["multi_blast64"]["network_error_held_out"] = network_error(runtime, w, mk)
    out["multi_blast64"]["workload"] = ("64 blasts (energy 0.02 in total) in the periodic 64^3 Sedov cube, "
                                        "background pressure 1e-2 (ic.multi_blast)")
    return out, w


def adaptive_section(runtime, cfg, p, tuning, args):
    """The same workload with per-particle smoothing lengths (adaptive_h):
    every step solves h_i <= H for an effective neighbour number of 32, H =
    1.25 kernelSize the search radius, and searches pairs with r < max(h_i,
    h_j).  Reports its throughput and the share of the h solve."""
    from dataclasses import replace
    cfg_a = replace(cfg, adaptive_h=True, n_ngb=32.0, kernel_size=cfg.kernel_size * 1.25)
    sim = runtime.Simulation(cfg_a, p)
    tuning_a = sim.autotune(2) if tuning else None
    st, _ = timed_steps(sim, args.warmup, args.steps)
    kt = kernel_breakdown(sim, args.steps)
    hs = sim.get("h_stats")
    h = sim.get("h")
    noi = sim.get("noi")
    sim.close()
    per = per_step(kt)
    return {"value": p.n * st.steps / (st.device_ms / 1e3), "ms_per_step": st.device_ms / st.steps,
            "n_ngb": 32.0, "search_radius_over_kernel_size": 1.25,
            "h_over_search_radius_mean": float(np.mean(h) / cfg_a.kernel_size),
            "neighbours_mean": float(np.mean(noi)),
            "h_solve_ms_per_step": per.get("smoothing_lengths"),
            "kernel_ms_per_step": per,
            "h_stats_last_solve": {"newton_iterations": float(hs[0]), "clamped": float(hs[1])},
            "tuning": tuning_a,
            "status": runtime.status_names(st.status)}


def ensemble_section(runtime, args, w_learned):
    """The 256-member Kelvin-Helmholtz ensemble (N log-uniform in [2500,
    40000], seeded): all members in one context, one CUDA graph per step,
    launch shapes and face-pass structure from the autotuner, with and
    without the learned guess; against the same members run one after
    another, each in its own context with the plain step.  Both sides are
    timed on the same clocks: host wall time around all timed steps (one
    synchronisation at each end), and the summed device time of the step
    calls (CUDA events)."""
    from meshlesshydro_gb300 import ic
    from meshlesshydro_gb300.config import MFVConfig
    members = ic.kh_ensemble(n_members=256, seed=7)
    cfg = MFVConfig.kelvin_helmholtz(members[0])
    npart = sum(m.n for m in members)
    clocks = ClockSampler(0)
    clocks.start()

    def batched(weights):
        sim = runtime.Simulation(cfg, members=members)
        if weights is not None:
            sim.set_pstar_weights(weights)
        tuning = sim.autotune(2)
        sim.set_graph_mode(True)
        st, wall = timed_steps(sim, args.warmup, args.steps)
        sim.close()
        return tuning, st, wall

    progress("ensemble: batched, plain")
    tun_p, st_p, wall_p = batched(None)
    progress("ensemble: batched, learned")
    tun_l, st_l, wall_l = batched(w_learned) if w_learned is not None else (None, None, None)
    progress("ensemble: members one after another")
    # members one after another: every member's step is a plain mlh_step(1)
    sims = [runtime.Simulation(MFVConfig.kelvin_helmholtz(m), m) for m in members]
    for s_ in sims:
        s_.step(args.warmup)
    import torch
    torch.cuda.synchronize()
    seq_dev = 0.0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for s_ in sims:
            seq_dev += s_.step(1).device_ms
    torch.cuda.synchronize()
    seq_wall = time.perf_counter() - t0
    for s_ in sims:
        s_.close()
    ck = clocks.stop()
    units = npart * args.steps
    out = {"members": len(members), "particles": npart, "steps": args.steps,
           "batched_graph_value": units / wall_p,
           "batched_graph_device_value": units / (st_p.device_ms / 1e3),
           "sequential_value": units / seq_wall,
           "sequential_device_value": units / (seq_dev / 1e3),
           "batched_over_sequential": (units / wall_p) / (units / seq_wall),
           "batched_over_sequential_device": seq_dev / st_p.device_ms,
           "clock": "wall: host time around all timed steps, synchronised at both ends, on both sides; device: "
                    "CUDA-event time of the step calls, summed over calls on the sequential side",
           "newton_iterations_per_face": st_p.newton_iterations / max(st_p.faces, 1),
           "tuning": tun_p, "clocks": ck, "status": runtime.status_names(st_p.status)}
    if st_l is not None:
        out.update({"learned_value": units / wall_l, "learned_device_value": units / (st_l.device_ms / 1e3),
                    "learned_over_plain": wall_p / wall_l,
                    "learned_over_sequential": (units / wall_l) / (units / seq_wall),
                    "learned_faces": int(st_l.learned_faces),
                    "learned_tuning": tun_l})
    return out


def run_mlh(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("gloo")
    else:
        dist = None
    from meshlesshydro_gb300 import build, runtime
    from meshlesshydro_gb300.replicas import gather_units, job_rate, job_seconds, replica_seed
    build.build()
    probe_clocks = ClockSampler(local)
    probe_clocks.start()
    progress("FP64 probe")
    fp64_peak, probe_mhz = runtime.probe_fp64_clock(1.0)
    progress("main workload: set-up and autotune")
    probe_ck = probe_clocks.stop()
    sm_count = torch.cuda.get_device_properties(local).multi_processor_count
    p, cfg = make_workload(args.workload, seed_offset=replica_seed(0, rank))
    ensemble = WORKLOADS[args.workload]["kind"] == "ensemble"
    members = p if ensemble else None
    sim = runtime.Simulation(cfg, members=members) if ensemble else runtime.Simulation(cfg, p)
    if ensemble:
        p = sim.host  # concatenated state: .n
    if args.tuning:
        sim.set_tuning(json.loads(args.tuning))
        tuning = json.loads(args.tuning)
    else:
        tuning = None if args.no_autotune else sim.autotune(2)
    progress(f"main workload: tuning {tuning}")
    sim.step(args.warmup)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    t0 = time.perf_counter()
    st = sim.step(args.steps)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    ck = clocks.stop()
    t_max = job_seconds(st.device_ms / 1e3, dist)
    faces_per_step = st.faces / max(st.steps, 1)
    pairs_per_step = st.pair_interactions / max(st.steps, 1)
    rho_plain = sim.get("rho")
    kt = kernel_breakdown(sim, args.steps)
    make_main = ((lambda: runtime.Simulation(cfg, members=members)) if ensemble
                 else (lambda: runtime.Simulation(cfg, p)))

    # end to end through the C ABI with host buffers: H2D of the state,
    # one step, D2H of the state, every step (pinned host memory)
    n = p.n
    keys = ("x", "y", "z", "vx", "vy", "vz", "m", "u")
    pinned = {k: torch.empty(n, dtype=torch.float64, pin_memory=True) for k in keys}
    view = runtime.ParticlesView()
    view.n = n
    for k in keys:
        setattr(view, k, ctypes.cast(pinned[k].data_ptr(), ctypes.POINTER(ctypes.c_double)))
    L = sim.L
    L.mlh_get_fields(sim.h, ctypes.byref(view))
    e2e_steps = max(2, min(args.steps, 5))
    used = 8 if cfg.dim == 3 else 6
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        L.mlh_set_fields(sim.h, ctypes.byref(view))
        sim.step(1)
        L.mlh_get_fields(sim.h, ctypes.byref(view))
    e2e_wall = job_seconds(time.perf_counter() - t0, dist)
    units = gather_units(n * st.steps, dist)
    sim.close()

    extra = {}
    w_learned = None
    main_kind = WORKLOADS[args.workload]["kind"]
    if not args.no_learned and main_kind in ("sedov", "multi_blast"):
        extra["learned"], w_learned = learned_section(runtime, args, make_main, tuning, st, kt, rho_plain)
    if not args.no_adaptive and main_kind == "sedov":
        progress("adaptive smoothing lengths")
        extra["adaptive_h"] = adaptive_section(runtime, cfg, p, tuning, args)
    if not args.no_ensemble and rank == 0:
        extra["ensemble"] = ensemble_section(runtime, args, w_learned)

    if rank != 0:
        if dist:
            dist.barrier()
        return 0
    value = job_rate(units, t_max)
    peaks, peak_kind = measured_peaks()
    ms_step = 1e3 * t_max / st.steps
    per = per_step(kt)
    # dominant kernel and its roofline on executed FP64 operations
    dom_name = max(per.items(), key=lambda kv: kv[1])[0]
    dom_launches, dom_ms = kt[dom_name]
    dom_avg_s = dom_ms / max(dom_launches, 1) / 1e3
    dim = cfg.dim
    unit = KERNEL_UNITS.get(dom_name, "particle")
    units_launch = faces_per_step if unit == "face" else float(n)
    fl, by = KERNEL_EXEC.get(dim, {}).get(dom_name, (None, None))
    achieved = fl * units_launch / dom_avg_s / 1e12 if fl else None
    step_ops = step_fp64(dim, float(n), faces_per_step) if dim in KERNEL_EXEC else None
    per_cycle_peak = probe_mhz * 1e6 * sm_count * FP64_OPS_PER_SM_CYCLE / 1e12 if probe_mhz else None
    roofline = {"kernel": f"{dom_name} (k_faces_block / k_faces)" if dom_name == "faces_riemann" else dom_name,
                "bound": "fp64", "unit": "TFLOP/s",
                "achieved": achieved, "peak": fp64_peak,
                "frac": (achieved / fp64_peak) if (achieved and fp64_peak) else None,
                "traffic": by * units_launch if by else None,
                "units": f"{unit}s", "units_per_launch": units_launch, "fp64_flops_per_unit": fl,
                "flops_source": "executed: FP64 operations the kernel executes per unit (ncu: 2 x DFMA + DADD + "
                                "DMUL thread instructions per unit, on the 64^3 Sedov step), not the reference's "
                                "operation count",
                "fp64_pipe_active_ncu": KERNEL_FP64_PIPE.get(dim, {}).get(dom_name),
                "fp64_instr_frac": ((KERNEL_FP64_INSTR[dim][dom_name] * units_launch / dom_avg_s) /
                                    (fp64_peak * 1e12 / 2.0))
                if (dom_name in KERNEL_FP64_INSTR.get(dim, {}) and fp64_peak) else None,
                "fp64_instr_frac_note": "FP64 thread instructions (DFMA + DADD + DMUL) per second over the probe's "
                                        "(its TFLOP/s / 2, all FMAs): the pipe's issue rate, where frac counts an "
                                        "FMA twice and an add or multiply once",
                "peak_source": "measured: FP64 FMA-chain probe (mlh_probe_fp64_clock) on this GPU in this run",
                "avg_launch_ms": dom_avg_s * 1e3,
                "hbm_view": {"achieved_gbs": (by * units_launch / dom_avg_s / 1e9) if by else None,
                             "peak_gbs": peaks.get("hbm_gbs"), "peak_source": peak_kind},
                "step_check": {"fp64_flops_per_step": step_ops,
                               "tflops": step_ops / (ms_step / 1e3) / 1e12 if step_ops else None,
                               "frac": (step_ops / (ms_step / 1e3) / 1e12 / fp64_peak) if step_ops else None,
                               "note": "every kernel's executed FP64 operations per step over ms_per_step; "
                                       "at most 1 (the kernels overlap only the integer face links)"}}
    try:   # every kernel against its roofline (arithmetic on the measured times)
        kernels = kernel_rooflines(per, dim, float(n), float(faces_per_step), fp64_peak, peaks.get("hbm_gbs"))
        kernels["source"] = ("ms: CUDA events; FP64 operations and DRAM bytes per unit: ncu captures of the same "
                             "kernels (3D Sedov 64^3, 2D KH ensemble members); peaks: FP64 FMA probe, measured "
                             "HBM copy")
    except Exception as exc:   # never let the breakdown cost the bench line
        kernels = {"error": repr(exc)}
    line = {"metric": METRIC, "value": value, "unit": "particle-updates/s", "n_gpus": ws, "steps": st.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "particles_per_gpu": n, "dim": cfg.dim,
                       "periodic": bool(cfg.periodic), "kernel_size": cfg.kernel_size,
                       "pair_interactions_per_step": pairs_per_step, "faces_per_step": faces_per_step,
                       "l2": "inputs larger than L2 (state + neighbour lists >> 129 MB)",
                       "parallelism": f"replicas x{ws}"},
            "pair_interactions_per_s": ws * pairs_per_step * st.steps / t_max,
            "newton_iterations_per_face": st.newton_iterations / max(st.faces, 1),
            "status": runtime.status_names(st.status),
            "wall_s_timed": wall,
            "gpu_launches": LAUNCHES_PER_STEP * st.steps,
            "kernel_ms_per_step": per,
            "kernel_ms_source": "up to 3 further steps with per-kernel CUDA events, which serialise the face-link "
                                "stream that the timed steps overlap with the time step and gradients",
            "roofline": roofline,
            "fp64_probe": {"tflops": fp64_peak, "sm_mhz": probe_mhz, "sm_count": sm_count,
                           "per_cycle_peak_tflops": per_cycle_peak,
                           "per_cycle_frac": fp64_peak / per_cycle_peak if per_cycle_peak else None,
                           "tflops_at_max_clock": (fp64_peak * probe_ck["sm_max_mhz"] / probe_mhz
                                                   if probe_mhz and probe_ck.get("sm_max_mhz") else None),
                           "clocks": probe_ck},
            "kernels": kernels,
            "clocks": ck,
            "tuning": tuning,
            **extra,
            "e2e": {"value": job_rate([u / st.steps * e2e_steps for u in units], e2e_wall),
                    "unit": "particle-updates/s",
                    "h2d_bytes_per_step": used * 8 * n, "d2h_bytes_per_step": used * 8 * n,
                    "steps": e2e_steps},
            "peaks": {"source": peak_kind, "hbm_gbs": peaks.get("hbm_gbs")}}
    if not args.no_cpu_baseline:
        progress("CPU baseline")
        line["cpu_baseline"] = cpu_baseline_sample(args.cpu_seconds,
                                                   "sedov" if main_kind in ("sedov", "multi_blast") else "kh")
    print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="mlh", choices=["mlh", "reference"])
    ap.add_argument("--workload", default="sedov128", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--tuning", default="", help="launch shapes as JSON (mlh_tuning fields) instead of the "
                                                 "autotuner's, e.g. for profiling")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned p* guess comparison")
    ap.add_argument("--no-adaptive", action="store_true", help="skip the per-particle smoothing-length run")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the 256-member KH ensemble comparison")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_mlh(args)


if __name__ == "__main__":
    sys.exit(main())
