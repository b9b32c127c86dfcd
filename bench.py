"""Throughput of the GB300 MFV step: particle-updates/s on one GB300.

Default workload: the 3D Sedov blast on a jittered 128^3 lattice (2,097,152
particles) in the periodic cube [-0.5, 0.5]^3, FP64 state, cubic spline with a
mean of 32 neighbours (kernelSize 2.102 lattice spacings), CFL 0.25, BETA 1,
pairwise limiter: the "plain GPU method at scale" configuration.  A step is one
full MFV step (binning, neighbour search, density, dt, gradients, limiter,
faces, exact Riemann solves, flux gather, kick/drift) over all particles.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl mlh|reference]
                    [--workload sedov128|sedov64|kh100]

Prints one JSON line.  --impl reference times the CPU restatement of the
reference's serial code (the oracle; the reference itself cannot run on the
GPU host) on a bounded sample of the same workload.
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
}
METRIC = "particle-updates/s per MFV step on 1 GB300"
# kernels launched by one plain mlh_step iteration (csrc/mlh_kernels.cu,
# launch_step; the ncu launch list of a step shows the same 20): binning
# (k_bounds_partial, k_bounds_final, k_assign, 3 scan kernels, k_fill_cells,
# k_sort_cells), k_neighbours, face links (3 scan kernels, k_link), k_timestep,
# k_dt_final, k_gradients, k_faces (first pass, second Newton pass), k_update,
# k_advance_time
LAUNCHES_PER_STEP = 20

# Algorithmic operations per canonical face of the dominant kernel (k_faces:
# effective face, face states, pairwise limiter, half-step prediction, exact
# Riemann solve, flux) in the reference's method, counted by the
# operation-counting build of the oracle (oracle/flops.py; every addition,
# multiplication, division, square root and pow weighs 1, an FMA 2) over 16
# steps: 3D on the 32^3 periodic Sedov lattice with the 128^3 workload's h/dx
# (1.28 Newton iterations per face), 2D on the 100x100 Kelvin-Helmholtz
# set-up (1.47).  The roofline's `achieved` uses these.
FACE_ALG_FLOPS = {3: 746.0, 2: 339.8}
# What k_faces (both passes, gamma = 5/3 path) executes per face, from ncu
# --set full captures: FP64 operations (2 x DFMA + DADD + DMUL thread
# instructions / faces) and DRAM bytes (read + write).  3D: the 64^3 periodic
# Sedov step; 2D: 32 members of the Kelvin-Helmholtz ensemble with the second
# Newton pass.
FACE_EXEC_FP64_FLOPS = {3: 541.0, 2: 391.0}
FACE_DRAM_BYTES = {3: 298.0, 2: 364.0}

# Every kernel of the step, per unit (particle, or canonical face for the
# face passes): (FP64 flops executed, DRAM bytes read + written) from the
# same ncu captures (3D: Sedov 64^3; 2D: 32 KH ensemble members), and the
# algorithmic operations of the reference's method from the
# operation-counting oracle (3D: 32^3 Sedov lattice; 2D: 100x100 KH set-up).
# The per-unit figures scale with the units of the measured workload.
KERNEL_UNITS = {"neighbours_density": "particle", "timestep": "particle", "gradients_limiter": "particle",
                "face_links": "particle", "faces_riemann": "face", "gather_update": "particle"}
KERNEL_EXEC = {
    3: {"neighbours_density": (1030.0, 917.0), "timestep": (607.0, 652.0), "gradients_limiter": (3747.0, 1692.0),
        "face_links": (0.0, 1010.0), "faces_riemann": (541.0, 298.0), "gather_update": (214.0, 1504.0)},
    2: {"neighbours_density": (597.0, 733.0), "timestep": (311.0, 748.0), "gradients_limiter": (1382.0, 1962.0),
        "face_links": (0.0, 781.0), "faces_riemann": (391.0, 364.0), "gather_update": (122.0, 915.0)},
}
KERNEL_ALG_OPS = {
    3: {"neighbours_density": 3618.0, "timestep": 754.0, "gradients_limiter": 7871.0, "face_links": 0.0,
        "faces_riemann": 746.0, "gather_update": 198.0},
    2: {"neighbours_density": 700.0, "timestep": 375.0, "gradients_limiter": 2678.0, "face_links": 0.0,
        "faces_riemann": 339.8, "gather_update": 108.0},
}


def kernel_rooflines(kernel_ms: dict, dim: int, particles: float, faces: float, fp64_peak_tflops, hbm_peak_gbs):
    """Each kernel of the step against the FP64 and the HBM roofline: its
    time per step (CUDA events), the FP64 flops it executes and the DRAM
    bytes it moves per unit (ncu), the rates they give, as fractions of the
    measured FP64 FMA peak and HBM copy bandwidth, and the rate of the
    reference's algorithmic operations."""
    out = {}
    for k, unit in KERNEL_UNITS.items():
        ms = kernel_ms.get(k)
        if not ms or ms <= 0.0 or dim not in KERNEL_EXEC:
            continue
        fl, by = KERNEL_EXEC[dim][k]
        alg = KERNEL_ALG_OPS[dim][k]
        units = faces if unit == "face" else particles
        s = ms / 1e3
        tf = fl * units / s / 1e12
        gbs = by * units / s / 1e9
        out[k] = {"ms_per_step": ms, "unit": unit, "units_per_step": units,
                  "fp64_flops_per_unit": fl, "fp64_tflops": tf,
                  "fp64_frac": tf / fp64_peak_tflops if fp64_peak_tflops else None,
                  "dram_bytes_per_unit": by, "hbm_gbs": gbs,
                  "hbm_frac": gbs / hbm_peak_gbs if hbm_peak_gbs else None,
                  "algorithmic_ops_per_unit": alg, "algorithmic_tflops": alg * units / s / 1e12}
    return out


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


def cpu_baseline_sample(seconds_hint: float = 20.0, kind: str = "sedov"):
    """The oracle (serial CPU restatement of the reference) on a bounded sample:
    whole MFV steps of the 32^3 Sedov lattice with the workload's particle
    density and neighbour count (same per-particle work as 128^3), or of the
    100x100 Kelvin-Helmholtz set-up for the 2D workloads."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from meshlesshydro_gb300 import ic
    from meshlesshydro_gb300.config import MFVConfig
    oracle.build()
    if kind == "sedov":
        p = ic.sedov(n_side=32, seed=2)
        cfg = MFVConfig.sedov(p, periodic=True)
        what = "32^3 periodic Sedov lattice"
    else:
        p = ic.kelvin_helmholtz(n_side=100, seed=1)
        cfg = MFVConfig.kelvin_helmholtz(p)
        what = "100x100 Kelvin-Helmholtz set-up"
    o = oracle.Oracle(cfg, p)
    o.step()  # warm-up
    steps, t0 = 0, time.perf_counter()
    while True:
        o.step()
        steps += 1
        el = time.perf_counter() - t0
        if el >= seconds_hint or steps >= 50:
            break
    return {"value": p.n * steps / el, "unit": "particle-updates/s", "cores": 1, "kind": "port",
            "sample": f"{steps} MFV steps of the {what} ({p.n} particles, the workload's h/dx and neighbour "
                      f"count), serial oracle, {el:.1f} s, host {cpu_model()}"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from meshlesshydro_gb300 import ic
    from meshlesshydro_gb300.config import MFVConfig
    oracle.build()
    w = WORKLOADS[args.workload]
    # bounded sample: the 32^3 lattice for Sedov workloads, the full KH set-up
    if w["kind"] == "sedov":
        p = ic.sedov(n_side=32, seed=2)
        cfg = MFVConfig.sedov(p, periodic=w["periodic"])
        sample = f"32^3 periodic Sedov lattice ({p.n} particles; same h/dx as {args.workload}), one MFV step per step"
    else:
        p = ic.kelvin_helmholtz(n_side=w["n_side"], seed=1)
        cfg = MFVConfig.kelvin_helmholtz(p)
        sample = f"{args.workload} ({p.n} particles), one MFV step per step"
    o = oracle.Oracle(cfg, p)
    for _ in range(args.warmup):
        o.step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.step()
    el = time.perf_counter() - t0
    val = p.n * args.steps / el
    line = {"metric": METRIC, "value": val, "unit": "particle-updates/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": args.workload, "sample": sample},
            "cpu_baseline": {"value": val, "unit": "particle-updates/s", "cores": 1, "kind": "port",
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


def learned_section(runtime, make_sim, tuning, args, faces_per_step, st_plain, kt_plain, rho_plain, ws, n):
    """The same steps with the learned p* guess: harvest faces of step 1
    (plain pipeline), train the MLP on 90 % of them, tune the learned
    pipeline's launch shapes and face-pass structure with the autotuner
    (which restores the state), step with the network guess to the same step
    count and compare with the plain run."""
    import torch
    sim2 = make_sim()
    if tuning:
        sim2.set_tuning(tuning)
    stride = max(1, int(faces_per_step // 2_000_000))
    t0 = time.perf_counter()
    x, t = sim2.harvest(stride=stride, capacity=int(faces_per_step // stride) + 64)
    rng = np.random.default_rng(0)
    perm = rng.permutation(x.shape[0])
    nval = x.shape[0] // 10
    val, tr = perm[:nval], perm[nval:]
    t1 = time.perf_counter()
    w, hist = runtime.pstar_train(x[tr], t[tr], epochs=20, batch=4096, lr=2e-3, seed=0)
    t2 = time.perf_counter()
    yv = runtime.pstar_infer(w, x[val])
    rel = np.abs(np.exp(yv.astype(np.float64) - t[val]) - 1.0)
    sim2.set_pstar_weights(w)
    tuning_l = sim2.autotune(2) if tuning else None
    if args.warmup > 1:
        sim2.step(args.warmup - 1)
    torch.cuda.synchronize()
    st = sim2.step(args.steps)
    rho = sim2.get("rho")
    kt = kernel_breakdown(sim2, args.steps)
    sim2.close()
    l1 = float(np.sum(np.abs(rho - rho_plain)) / np.sum(np.abs(rho_plain)))
    return {"value": ws * n * st.steps / (st.device_ms / 1e3),
            "plain_value": ws * n * st_plain.steps / (st_plain.device_ms / 1e3),
            "newton_iterations_per_face": st.newton_iterations / max(st.faces, 1),
            "plain_newton_iterations_per_face": st_plain.newton_iterations / max(st_plain.faces, 1),
            "fallback_rate": st.newton_fallbacks / max(st.learned_faces, 1),
            "learned_face_fraction": st.learned_faces / max(st.faces, 1),
            "faces_kernel_ms_per_step": kt["faces_riemann"][1] / max(kt["faces_riemann"][0], 1),
            "plain_faces_kernel_ms_per_step": kt_plain["faces_riemann"][1] / max(kt_plain["faces_riemann"][0], 1),
            "density_L1_vs_plain": l1,
            "tuning": tuning_l,
            "status": runtime.status_names(st.status),
            "guess": "p_TR * exp(y) where |y| > 0.01, else p_TR (two-rarefaction)",
            "train": {"samples": int(tr.size), "val_samples": int(nval), "harvest_stride": stride,
                      "harvest_step": 1, "epochs": 20, "batch": 4096, "lr": 2e-3,
                      "loss_first_epoch": float(hist[0]), "loss_last_epoch": float(hist[-1]),
                      "val_median_rel_err": float(np.median(rel)) if nval else None,
                      "val_p90_rel_err": float(np.quantile(rel, 0.9)) if nval else None,
                      "harvest_s": t1 - t0, "train_s": t2 - t1}}


def adaptive_section(runtime, cfg, p, tuning, args, ws):
    """The same workload with per-particle smoothing lengths (adaptive_h):
    every step solves h_i <= H for an effective neighbour number of 32, H =
    1.25 kernelSize the search radius, and searches pairs with r < max(h_i,
    h_j).  Reports its throughput and the share of the h solve."""
    import torch
    from dataclasses import replace
    cfg_a = replace(cfg, adaptive_h=True, n_ngb=32.0, kernel_size=cfg.kernel_size * 1.25)
    sim = runtime.Simulation(cfg_a, p)
    # its own launch shapes: the wider search radius changes the best ones
    tuning_a = sim.autotune(2) if tuning else None
    sim.step(args.warmup)
    torch.cuda.synchronize()
    st = sim.step(args.steps)
    kt = kernel_breakdown(sim, args.steps)
    hs = sim.get("h_stats")
    h = sim.get("h")
    noi = sim.get("noi")
    sim.close()
    per = {k: v[1] / max(v[0], 1) for k, v in kt.items()}
    return {"value": ws * p.n * st.steps / (st.device_ms / 1e3), "ms_per_step": st.device_ms / st.steps,
            "n_ngb": 32.0, "search_radius_over_kernel_size": 1.25,
            "h_over_search_radius_mean": float(np.mean(h) / cfg_a.kernel_size),
            "neighbours_mean": float(np.mean(noi)),
            "h_solve_ms_per_step": per.get("smoothing_lengths"),
            "kernel_ms_per_step": per,
            "h_stats_last_solve": {"newton_iterations": float(hs[0]), "clamped": float(hs[1])},
            "tuning": tuning_a,
            "status": runtime.status_names(st.status)}


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
    fp64_peak = runtime.probe_fp64_tflops(0.5)
    p, cfg = make_workload(args.workload, seed_offset=replica_seed(0, rank))
    ensemble = WORKLOADS[args.workload]["kind"] == "ensemble"
    members = p if ensemble else None
    sim = runtime.Simulation(cfg, members=members) if ensemble else runtime.Simulation(cfg, p)
    if ensemble:
        p = sim.host  # concatenated state: .n
    tuning = None if args.no_autotune else sim.autotune(2)
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
    rho_plain = sim.get("rho")      # density of step warmup + steps (autotune restored its trials)
    kt = kernel_breakdown(sim, args.steps)
    make_sim = ((lambda: runtime.Simulation(cfg, members=members)) if ensemble
                else (lambda: runtime.Simulation(cfg, p)))

    extra = {}
    if ensemble:
        # the same steps in graph mode (one CUDA graph per step), and the
        # members run one after another as separate plain simulations
        sim.set_graph_mode(True)
        sim.step(1)
        torch.cuda.synchronize()
        stg = sim.step(args.steps)
        graph_value = ws * p.n * stg.steps / (stg.device_ms / 1e3)
        sim.set_graph_mode(False)
        seq_steps = 2
        from meshlesshydro_gb300.config import MFVConfig
        sims = [runtime.Simulation(MFVConfig.kelvin_helmholtz(m), m) for m in members]
        for s_ in sims:
            s_.step(1)
        torch.cuda.synchronize()
        t0s = time.perf_counter()
        for _ in range(seq_steps):
            for s_ in sims:
                s_.step(1)
        torch.cuda.synchronize()
        seq_wall = time.perf_counter() - t0s
        seq_value = p.n * seq_steps / seq_wall
        del sims
        extra = {"ensemble": {"members": len(members), "particles": p.n,
                              "batched_graph_value": graph_value,
                              "sequential_value": seq_value,
                              "sequential": "each member its own context, one mlh_step(1) call per member per step, "
                                            f"{seq_steps} steps, wall clock",
                              "batched_over_sequential": graph_value / seq_value}}

    if not args.no_learned:
        extra["learned"] = learned_section(runtime, make_sim, tuning, args, faces_per_step, st, kt, rho_plain, ws, p.n)
    if not args.no_adaptive and WORKLOADS[args.workload]["kind"] == "sedov":
        extra["adaptive_h"] = adaptive_section(runtime, cfg, p, tuning, args, ws)

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
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        L.mlh_set_fields(sim.h, ctypes.byref(view))
        sim.step(1)
        L.mlh_get_fields(sim.h, ctypes.byref(view))
    e2e_wall = job_seconds(time.perf_counter() - t0, dist)
    units = gather_units(n * st.steps, dist)

    if rank != 0:
        if dist:
            dist.barrier()
        return 0
    value = job_rate(units, t_max)
    peaks, peak_kind = measured_peaks()
    # dominant kernel and its roofline
    dom = max(kt.items(), key=lambda kv: kv[1][1])
    dom_name, (dom_launches, dom_ms) = dom
    dom_avg_s = dom_ms / max(dom_launches, 1) / 1e3
    flops_per_face = FACE_ALG_FLOPS.get(cfg.dim)
    exec_per_face = FACE_EXEC_FP64_FLOPS.get(cfg.dim)
    bytes_per_face = FACE_DRAM_BYTES.get(cfg.dim)
    achieved_tf = (flops_per_face * faces_per_step / dom_avg_s / 1e12
                   if (dom_name == "faces_riemann" and flops_per_face) else None)
    exec_tf = (exec_per_face * faces_per_step / dom_avg_s / 1e12
               if (dom_name == "faces_riemann" and exec_per_face) else None)
    roofline = {"kernel": "k_faces (faces_riemann)" if dom_name == "faces_riemann" else dom_name,
                "bound": "fp64", "unit": "TFLOP/s",
                "achieved": achieved_tf, "peak": fp64_peak,
                "frac": (achieved_tf / fp64_peak) if (achieved_tf and fp64_peak) else None,
                "traffic": bytes_per_face * faces_per_step if bytes_per_face else None,
                "peak_source": "measured: FP64 FMA-chain probe (mlh_probe_fp64_tflops) on this GPU in this run",
                "units": "canonical faces", "units_per_launch": faces_per_step,
                "flops_per_unit": flops_per_face,
                "flops_source": "algorithmic: operations of the reference's method per canonical face, "
                                "counted by the operation-counting oracle (oracle/flops.py), each 1, an FMA 2",
                "executed": {"flops_per_unit": exec_per_face, "achieved": exec_tf,
                             "frac": (exec_tf / fp64_peak) if (exec_tf and fp64_peak) else None,
                             "source": "FP64 flops k_faces executes per face (ncu, 2 x DFMA + DADD + DMUL)"},
                "avg_launch_ms": dom_avg_s * 1e3,
                "hbm_view": {"achieved_gbs": (bytes_per_face * faces_per_step / dom_avg_s / 1e9) if bytes_per_face else None,
                             "peak_gbs": peaks.get("hbm_gbs"), "peak_source": peak_kind}}
    try:   # every kernel against its roofline (arithmetic on the measured times)
        kernels = kernel_rooflines({k: v[1] / max(v[0], 1) for k, v in kt.items()}, cfg.dim, float(n),
                                   float(faces_per_step), fp64_peak, peaks.get("hbm_gbs"))
        kernels["source"] = ("ms: CUDA events; FP64 flops and DRAM bytes per unit: ncu --set full of the same "
                             "kernels (3D Sedov 64^3, 2D KH ensemble members); algorithmic operations: "
                             "operation-counting oracle; peaks: FP64 FMA probe, measured HBM copy")
    except Exception as exc:   # never let the breakdown cost the bench line
        kernels = {"error": repr(exc)}
    line = {"metric": METRIC, "value": value, "unit": "particle-updates/s", "n_gpus": ws, "steps": st.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_max / st.steps, "higher_is_better": True,
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
            "kernel_ms_per_step": {k: v[1] / max(v[0], 1) for k, v in kt.items()},
            "kernel_ms_source": "up to 3 further steps with per-kernel CUDA events, which serialise the face-link "
                                "stream that the timed steps overlap with the time step and gradients",
            "roofline": roofline,
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
        line["cpu_baseline"] = cpu_baseline_sample(args.cpu_seconds,
                                                   "sedov" if WORKLOADS[args.workload]["kind"] == "sedov" else "kh")
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
    ap.add_argument("--no-learned", action="store_true", help="skip the learned p* guess comparison")
    ap.add_argument("--no-adaptive", action="store_true", help="skip the per-particle smoothing-length run")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_mlh(args)


if __name__ == "__main__":
    sys.exit(main())
