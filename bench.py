#!/usr/bin/env python
"""Benchmark of the GB300 implicit tet-FEM timestep (BACKWARD_EULER_VELOCITY).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl ours|reference]

One "step" is one BACKWARD_EULER_VELOCITY::solve over the workload (all scenes
of a batch).  Prints ONE JSON line (rank 0).  `value` is device-resident
steps/s over the timed region (CUDA events on the library's stream, W warm-up
steps first); `e2e` is the same metric through the public API with host
buffers (pinned) copied in and out every step.  `--impl reference` times the
CPU restatement of the reference algorithm (oracle/) on the host cores for the
same workload.

Workloads (synthetic, seeded; see hobakv1_gb300/scenes.py):
  kuhn40_snh_twist        40^3 Kuhn cube, 384,000 tets, SNH E=1e4 nu=0.45, compressed 0.6 + twisted, FP64
  kuhn40_arap_twist       same with ARAP
  kuhn40_snh_twist_mixed  the SNH case with FP32 Hessian/SpMV/inner PCG and FP64 refinement
  kuhn10_snh              10^3 Kuhn cube, 6,000 tets, SNH E=1e3 nu=0.45 (the CPU-runnable case)
  mix256_mixed            256 scenes, N ~ U{6..24} cells per side, SNH/ARAP, mu log-uniform,
                          one batched mixed-precision step = every scene advanced once
  mix256_fp64             the same mix batched in FP64
  mix64_mixed             the first 64 scenes of the mix, mixed (a profiling-sized case)
  kuhn40_snh_twist_position[_mixed], mix256_position_mixed
                          the same inputs stepped by BACKWARD_EULER_POSITION (Rayleigh damped)
  kuhn40_snh_hang_newmark[_mixed], mix256_newmark_mixed
                          NEWMARK (a Newton loop of solves per step) on the top-pinned 40^3
                          cube under gravity and on the mix
  serve_poisson           continuous batching: 32 jobs (N ~ U{8..32}, 10-200 steps, half two cubes in
                          vertex-face contact) arriving as a Poisson stream at 50, 400 and 2000 jobs/s,
                          mixed precision and plain FP64; job-steps/s, p50/p99 step and job latency
  two_cubes24_contact_position[_mixed]
                          two 24^3 cubes in self contact (vertex-face and edge-edge, distance 1e-2),
                          BACKWARD_EULER_POSITION
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "steps/s, p50/p99 step latency: batched mixed-precision vs plain FP64, same tol"
WORKLOADS = {
    "kuhn40_snh_twist": dict(kind="config2", N=40, material="snh", precision=0),
    "kuhn40_arap_twist": dict(kind="config2", N=40, material="arap", precision=0),
    "kuhn40_snh_twist_mixed": dict(kind="config2", N=40, material="snh", precision=1),
    "kuhn10_snh": dict(kind="config1", N=10, material="snh", precision=0),
    "mix256_mixed": dict(kind="mix", count=256, material="snh/arap", precision=1),
    "mix256_fp64": dict(kind="mix", count=256, material="snh/arap", precision=0),
    "mix64_mixed": dict(kind="mix", count=64, material="snh/arap", precision=1),
    # every third scene of the 256-scene mix (86 scenes, ~2 GB on the device): profiling case
    "mix86_mixed": dict(kind="mix", count=256, stride=3, material="snh/arap", precision=1),
    # BACKWARD_EULER_POSITION (Rayleigh damped, alpha = beta = 0.01) on the same inputs
    "kuhn40_snh_twist_position": dict(kind="config2", N=40, material="snh", precision=0, integrator="position"),
    "kuhn40_snh_twist_position_mixed": dict(kind="config2", N=40, material="snh", precision=1,
                                            integrator="position"),
    "mix256_position_mixed": dict(kind="mix", count=256, material="snh/arap", precision=1, integrator="position"),
    # NEWMARK (a Newton loop of linear solves per step; undamped, since the
    # reference zeroes its C: on the released compressed-and-twisted cube its
    # Newton loop fails at 40^3 and the reference run diverges, so the 40^3
    # case is the top-pinned cube hanging under gravity)
    "kuhn40_snh_hang_newmark": dict(kind="config1", N=40, material="snh", precision=0, integrator="newmark"),
    "kuhn40_snh_hang_newmark_mixed": dict(kind="config1", N=40, material="snh", precision=1, integrator="newmark"),
    "mix256_newmark_mixed": dict(kind="mix", count=256, material="snh/arap", precision=1, integrator="newmark"),
    "serve_poisson": dict(kind="serve", count=32, lambdas=[50, 400, 2000], material="snh/arap",
                          precision=1),
    # self contact: two 24^3 cubes resting on each other (62,500 vertices),
    # vertex-face and edge-edge collisions at distance 1e-2, position integrator
    "two_cubes24_contact_position_mixed": dict(kind="contact", N=24, material="snh", precision=1,
                                               integrator="position",
                                               contact=dict(vf=True, ee=True, eps=1e-2, mu=1e3, beta=1e-3)),
    "two_cubes24_contact_position": dict(kind="contact", N=24, material="snh", precision=0, integrator="position",
                                         contact=dict(vf=True, ee=True, eps=1e-2, mu=1e3, beta=1e-3)),
}
# the metric's headline: batched mixed precision on the 256-scene mix, with the
# plain (unbatched) FP64 GPU path measured beside it
DEFAULT_WORKLOAD = "mix256_mixed"


def make_scenes(spec):
    from hobakv1_gb300 import scenes
    if spec["kind"] == "config2":
        return [scenes.config2_scene(spec["N"], spec["material"])]
    if spec["kind"] == "config1":
        return [scenes.config1_scene(spec["N"], spec["material"])]
    if spec["kind"] == "mix":
        return scenes.config4_scenes(spec["count"])[::spec.get("stride", 1)]
    if spec["kind"] == "serve":
        return scenes.config5_jobs(spec["count"])
    if spec["kind"] == "contact":
        return [scenes.two_cubes_scene(spec["N"])]
    raise ValueError(spec)


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None, "samples": len(sm), "reasons": sorted(reasons)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(workload):
    """DRAM bytes per launch of each kernel from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(path):
        return {}
    with open(path) as f:
        return json.load(f).get(workload, {})


def cpu_baseline(scene_list, steps, warmup, max_scenes=16, integrator="velocity", contact=None):
    """The oracle (CPU restatement of the reference algorithm, OpenMP on all
    host cores) on the same workload; bounded sample.  Large mixes time a
    seeded subset (every k-th scene) and scale by scene count.
    Returns (steps/s of the whole workload, per-step seconds, cores, sample)."""
    from oracle import oracle
    oracle.build()
    stride = max(1, -(-len(scene_list) // max_scenes))
    subset = scene_list[::stride]
    scale = len(scene_list) / len(subset)
    sims = [oracle.Sim(s, precond=0, integrator=integrator) for s in subset]
    if contact:
        for sim in sims:
            sim.set_collisions(contact["vf"], contact["eps"], contact["mu"], contact["beta"], ee=contact["ee"])
    if warmup:
        for sim in sims:
            sim.step(warmup)
    lat = []
    for _ in range(steps):
        ts = time.perf_counter()
        for sim in sims:
            sim.step(1)
        lat.append((time.perf_counter() - ts) * scale)
    value = steps / sum(lat)
    sample = (f"{steps} steps of {len(subset)} of {len(scene_list)} scene(s) (every {stride}th), "
              f"time scaled by {scale:.1f}" if stride > 1 else f"{steps} steps of all {len(scene_list)} scene(s)")
    return value, lat, oracle.lib().oracle_threads(), sample


def plain_fp64_gpu(scene_list, steps, integrator=0):
    """The plain FP64 GPU path on a mix: every scene as its own batch, one
    after another (no batching), same tolerance.  Returns mix steps/s."""
    import torch
    from hobakv1_gb300 import hobak
    batches = [hobak.BATCH([s], hobak.solver_opts(precision=hobak.PRECISION_FP64, integrator=integrator))
               for s in scene_list]
    for b in batches:
        b.step(1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        for b in batches:
            b.step(1)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    for b in batches:
        b.close()
    return steps / dt


def batched_fp64_gpu(scene_list, steps, warmup, integrator, no_autotune):
    """The same mix as one FP64 batch: steps/s and ms per step (CUDA events)."""
    import torch
    from hobakv1_gb300 import hobak
    b = hobak.BATCH(scene_list, hobak.solver_opts(precision=hobak.PRECISION_FP64, integrator=integrator))
    tune = b.get_tuning() if no_autotune else b.autotune(reps=1)
    b.step(max(warmup, 1))
    stream = torch.cuda.ExternalStream(b.stream_handle())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        b.step(1)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    b.close()
    return 1e3 / ms, ms, tune


def cpu_model() -> str:
    """The host CPU's model name (/proc/cpuinfo), or the machine type."""
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                key = line.split(":")[0].strip().lower()
                if key in ("model name", "cpu model", "hardware"):
                    return line.split(":", 1)[1].strip()
        import platform
        return platform.machine() + " (no model name in /proc/cpuinfo)"
    except OSError:
        import platform
        return platform.machine()


def port_vs_reference():
    """Speed of the oracle port against the reference built from its sources,
    measured side by side on the x86 build host (oracle/port_vs_reference.py),
    where the reference compiles; the reference's x86 build cannot run here."""
    path = os.path.join(ROOT, "oracle", "port_vs_reference.json")
    if not os.path.exists(path):
        return {}
    with open(path) as f:
        m = json.load(f)
    return {"port_speed_vs_reference": m.get("port_speed_vs_reference"),
            "port_vs_reference_how": m.get("how")}


def serve_once(job_specs, arrivals, precision, budget_bytes, tuning=None, impl="native"):
    """Drive the continuous-batching server (the library's own, or the Python
    one) with jobs arriving at the given times (seconds from start).  Returns
    (wall seconds, jobs, server)."""
    from hobakv1_gb300 import serving
    cls = serving.NativeServer if impl == "native" else serving.Server
    srv = cls(budget_bytes, precision=precision, async_build=True, max_admit_per_tick=8, tuning=tuning)
    jobs = [serving.Job(k, sc, n, contact) for k, (sc, n, contact) in enumerate(job_specs)]
    t0 = time.perf_counter()
    i = 0
    while i < len(jobs) or not srv.idle():
        now = time.perf_counter() - t0
        while i < len(jobs) and arrivals[i] <= now:
            srv.submit(jobs[i])
            i += 1
        if srv.idle():
            if i < len(jobs):
                time.sleep(max(0.0, arrivals[i] - (time.perf_counter() - t0)))
            continue
        srv.pump()
    wall = time.perf_counter() - t0
    srv.close()
    return wall, jobs, srv


def run_serving(args, spec, job_specs):
    """Poisson arrivals at each rate of `lambdas`, mixed precision and plain
    FP64, the same seeded jobs; p50/p99 of step latency (the tick each job-step
    ran in) and of job latency (arrival to result on the host); job-steps/s
    over the wall time; the mixed result's position error against FP64."""
    import torch
    torch.cuda.set_device(0)
    from hobakv1_gb300 import hobak
    rng = np.random.default_rng(20261203 + 7)
    gaps = rng.exponential(1.0, len(job_specs))
    total_steps = sum(n for _, n, _ in job_specs)
    budget = int(float(spec.get("budget_gb", 64)) * (1 << 30))
    # cohorts solve their small scenes in clusters (contact scenes included)
    # unless --cluster-pcg 0
    serve_tuning = {"cluster_pcg": 1 if args.cluster_pcg is None else args.cluster_pcg}
    # warm the library (module load, first graph capture) outside the timing
    serve_once(job_specs[:2], [0.0, 0.0], hobak.PRECISION_MIXED, budget, impl=args.serve_impl)
    runs = {}
    finals = {}
    for prec_name, prec in (("mixed", hobak.PRECISION_MIXED), ("fp64", hobak.PRECISION_FP64)):
        for lam in spec["lambdas"]:
            arrivals = np.cumsum(gaps) / lam
            wall, jobs, srv = serve_once(job_specs, arrivals, prec, budget, serve_tuning, args.serve_impl)
            step_ms = [ms for j in jobs for ms in j.step_ms]
            job_s = [j.finished - j.submitted for j in jobs]
            runs[f"{prec_name}@{lam}"] = {
                "lambda_per_s": lam, "precision": prec_name, "job_steps_per_s": total_steps / wall,
                "wall_s": wall, "step_p50_ms": float(np.percentile(step_ms, 50)),
                "step_p99_ms": float(np.percentile(step_ms, 99)),
                "job_p50_s": float(np.percentile(job_s, 50)), "job_p99_s": float(np.percentile(job_s, 99)),
                "ticks": srv.ticks}
            finals[(prec_name, lam)] = [j.result_x + j.scene.rest.reshape(-1) for j in jobs]
    lam_hi = max(spec["lambdas"])
    errs = [np.linalg.norm(a - b) / np.linalg.norm(b)
            for a, b in zip(finals[("mixed", lam_hi)], finals[("fp64", lam_hi)])]
    contact = [c is not None for _, _, c in job_specs]
    err_contact = [e for e, c in zip(errs, contact) if c]
    err_free = [e for e, c in zip(errs, contact) if not c]
    hi_m, hi_f = runs[f"mixed@{lam_hi}"], runs[f"fp64@{lam_hi}"]
    nbytes_in = sum(sc.nv * 3 * 8 * 2 + sc.nt * 16 + sc.nv * 24 for sc, _, _ in job_specs)
    nbytes_out = sum(sc.nv * 3 * 8 * 2 for sc, _, _ in job_specs)
    line = {"metric": METRIC, "value": hi_m["job_steps_per_s"], "unit": "job-steps/s", "n_gpus": 1,
            "steps": total_steps, "warmup": 1, "ms_per_step": 1e3 / hi_m["job_steps_per_s"],
            "p50_ms": hi_m["step_p50_ms"], "p99_ms": hi_m["step_p99_ms"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": args.workload, "jobs": len(job_specs), "lambdas_per_s": spec["lambdas"],
                       "cells_per_side": "U{8..32}", "steps_per_job": "U{10..200}",
                       "contact": "even jobs: two SNH cubes, vertex-face eps 1e-3, stiffness 1e3, beta 1e-3",
                       "tets_total": int(sum(sc.nt for sc, _, _ in job_specs)), "pcg_tol": 1e-8,
                       "budget_gb": budget / (1 << 30),
                       "server": ("hobak_server_* (the library's native server)" if args.serve_impl == "native"
                                  else "serving.Server (Python)"),
                       "timing": "wall clock from the first arrival to the last result on the host",
                       "pcg_path": ("cluster-resident for scenes that fit 16 CTAs, tile path for larger ones"
                                    if serve_tuning["cluster_pcg"] else "tile path")},
            "serving": runs,
            "mixed_over_fp64_at_max_lambda": hi_m["job_steps_per_s"] / hi_f["job_steps_per_s"],
            "mixed_vs_fp64_rel_pos_err": {
                "max": float(max(errs)), "median": float(np.median(errs)),
                "max_without_contact": float(max(err_free)) if err_free else None,
                "max_with_contact": float(max(err_contact)) if err_contact else None,
                "worst_job": int(np.argmax(errs)),
                "per_job": [float(e) for e in errs]},
            "e2e": {"value": hi_m["job_steps_per_s"], "unit": "job-steps/s", "h2d_bytes_per_step":
                    nbytes_in / total_steps, "d2h_bytes_per_step": nbytes_out / total_steps,
                    "api": ("hobak_server_submit/pump/job" if args.serve_impl == "native"
                    else "serving.Server over hobak_batch_create/step_async/wait/get_state")}}
    print(json.dumps(line), flush=True)


def run_reference(args, spec, scene_list):
    """The reference algorithm on the host cores: the oracle port (the x86
    reference build cannot run on this host) on every scene of the workload,
    W warm-up steps then exactly K timed steps, each a full step of the whole
    workload (no subset, no extrapolation); plus a 1-thread figure on a
    sample of the scenes."""
    rank, world, _ = dist_info()
    if rank != 0:
        return
    from oracle import oracle
    oracle.build()
    integrator = spec.get("integrator", "velocity")
    contact = spec.get("contact")
    sims = [oracle.Sim(s, precond=0, integrator=integrator) for s in scene_list]
    if contact:
        for sim in sims:
            sim.set_collisions(contact["vf"], contact["eps"], contact["mu"], contact["beta"], ee=contact["ee"])
    cores = oracle.set_threads(0)
    for _ in range(args.warmup):
        for sim in sims:
            sim.step(1)
    lat = []
    for _ in range(args.steps):
        ts = time.perf_counter()
        for sim in sims:
            sim.step(1)
        lat.append(time.perf_counter() - ts)
    value = args.steps / sum(lat)
    # 1 thread against all threads on the same sample (every k-th scene, one step)
    stride = max(1, len(sims) // 16)
    sample = sims[::stride]
    t_all = time.perf_counter()
    for sim in sample:
        sim.step(1)
    t_all = time.perf_counter() - t_all
    oracle.set_threads(1)
    t_one = time.perf_counter()
    for sim in sample:
        sim.step(1)
    t_one = time.perf_counter() - t_one
    oracle.set_threads(0)
    lat_ms = [1e3 * x for x in lat]
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / value,
            "p50_ms": float(np.percentile(lat_ms, 50)), "p99_ms": float(np.percentile(lat_ms, 99)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": args.workload, **config_of(spec, scene_list)},
            "preconditioner": "jacobi (Eigen DiagonalPreconditioner, the reference's)",
            "cpu_baseline": {"value": value, "unit": "steps/s", "cores": cores, "kind": "port",
                             "sample": f"every step of all {len(sims)} scene(s): {args.warmup} warm-up steps, "
                                       f"then {args.steps} timed steps from the workload's initial state",
                             "cpu_model": cpu_model(),
                             "one_thread": {"sample": f"one step of {len(sample)} of the {len(sims)} scene(s) "
                                                      f"(every {stride}th), after the timed steps",
                                            "ms_1_thread": 1e3 * t_one, f"ms_{cores}_threads": 1e3 * t_all,
                                            "thread_speedup": t_one / t_all if t_all > 0 else None},
                             **port_vs_reference()},
            "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_reference_serving(args, spec, job_specs, sample_jobs=4, steps=2):
    """The oracle on the serving mix: a bounded sample (the first jobs, each
    `steps` steps from its initial state, contact on where the job has it),
    run one after another on the host cores; job-steps/s."""
    if dist_info()[0] != 0:
        return
    from oracle import oracle
    oracle.build()
    sims = []
    for sc, _, contact in job_specs[:sample_jobs]:
        sim = oracle.Sim(sc, precond=0)
        if contact is not None:
            sim.set_collisions(True, *contact)
        sims.append(sim)
    t0 = time.perf_counter()
    for sim in sims:
        sim.step(steps)
    value = steps * len(sims) / (time.perf_counter() - t0)
    sample = (f"{steps} steps of each of the first {len(sims)} of {len(job_specs)} jobs "
              f"({sum(s.scene.nt for s in sims)} tets), one after another")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "job-steps/s", "n_gpus": args.gpus,
            "steps": steps * len(sims), "warmup": 0, "ms_per_step": 1e3 / value, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "jobs": len(job_specs)},
            "cpu_baseline": {"value": value, "unit": "job-steps/s", "cores": oracle.lib().oracle_threads(),
                             "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "job-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def config_of(spec, scene_list):
    nt = int(sum(s.nt for s in scene_list))
    hess_mb = nt * 90 * (8 if spec["precision"] == 0 else 4) / 1e6
    return {"scenes": len(scene_list), "tets": nt, "verts": int(sum(s.nv for s in scene_list)),
            "material": spec["material"], "precision": "fp64" if spec["precision"] == 0 else "mixed",
            "integrator": {"position": "BACKWARD_EULER_POSITION (Rayleigh alpha = beta = 0.01)",
                           "newmark": "NEWMARK (beta 1/4, gamma 1/2, Newton to |rhs|^2 <= 1e-7, at most 10)"}
                          .get(spec.get("integrator"), "BACKWARD_EULER_VELOCITY"),
            **({"contact": {"vertex_face": spec["contact"]["vf"], "edge_edge": spec["contact"]["ee"],
                            "eps": spec["contact"]["eps"], "stiffness": spec["contact"]["mu"],
                            "damping_beta": spec["contact"]["beta"]}} if spec.get("contact") else {}),
            "pcg_tol": 1e-8, "pcg_max_iters": 1000,
            "l2": f"each step writes {hess_mb:.0f} MB of element Hessians (> 129 MB L2 at 40^3 and the mix); "
                  "no explicit flush"}


# GB300 issues FP64 at 2 thread-instructions per SM per clock (ncu:
# sm__sass_thread_inst_executed_op_dfma_pred_on.sum.peak_sustained = 304 over
# 152 SMs), 1/64 of the FP32 rate.
FP64_PER_SM_CLK = 2
NUM_SMS = 152


def step_rooflines(batch, spec, scene_list, phases, phase_steps, iters_by_scene, workload, sm_mhz):
    """Rooflines of the kernels the timed step launches.

    element, assembly: k_element / k_assemble, one launch each per step
      (velocity and position integrators): algorithmic bytes per launch
      (hobak_batch_kernel_bytes) over the CUDA-event launch time
      (hobak_batch_time_kernels), against the measured HBM copy bandwidth;
      the element kernel also against the FP64 pipe, from the ncu count of
      its FP64 thread-instructions on this workload (profiles/traffic.json).
    pcg: the step's inner solves, every refinement sweep, on whichever path
      each scene takes (thread-block clusters, or the tile path's SpMV and
      update kernels): per scene, PCG iterations x the bytes one iteration
      streams (the tile path's SpMV + update bytes of that scene), summed over
      scenes, over the phase's CUDA-event time per step.
    spmv, pcg_update: the tile-path kernels timed over the whole batch; the
      step launches them only for scenes on the tile path."""
    kms = batch.time_kernels(reps=10)
    kbytes = batch.kernel_bytes()
    peak, peak_kind = measured_peaks()
    traffic = ncu_traffic(workload)
    w = 4.0 if spec["precision"] == 1 else 8.0
    paths = batch.pcg_path()
    n_tile = int((paths == 0).sum())
    phase_ms = {k: v[0] / phase_steps for k, v in phases.items()}
    newmark = spec.get("integrator") == "newmark"
    gbs = lambda nbytes, ms: nbytes / (ms * 1e-3) / 1e9
    ent = {}
    for k, name in (("element", "k_element<float>" if w == 4 else "k_element<double>"),
                    ("assemble", "k_assemble<float>" if w == 4 else "k_assemble<double>")):
        a = gbs(kbytes[k], kms[k])
        ent[k] = {"kernel": name, "launch_ms": kms[k], "algorithmic_bytes": kbytes[k], "GB/s": a,
                  "frac_hbm": a / peak, "traffic": traffic.get(k),
                  "step_ms": phase_ms["element" if k == "element" else "assembly"],
                  "launches_per_step": None if newmark else 1}
    fp64_inst = traffic.get("fp64_inst_element")
    if fp64_inst and sm_mhz:
        rate = fp64_inst / (kms["element"] * 1e-3)
        fpeak = FP64_PER_SM_CLK * NUM_SMS * sm_mhz * 1e6
        ent["element"]["fp64"] = {"inst_per_launch": fp64_inst, "inst_per_s": rate, "peak_inst_per_s": fpeak,
                                  "frac": rate / fpeak, "clock_mhz": sm_mhz,
                                  "how": "ncu FP64 thread-instructions (dadd + dmul + dfma) of one launch on this "
                                         "workload, over the live launch time; peak 2 per SM per clock"}
    # per-scene bytes one PCG iteration streams: the tile path's SpMV (blocks
    # + columns, rowptr, u gathered, w written) and update (42 values per vertex)
    per_iter = np.array([batch.blocks(i) * (9 * w + 4) + s.nv * (4 + 6 * w) + s.nv * w * 42
                         for i, s in enumerate(scene_list)])
    pcg_bytes = float((iters_by_scene * per_iter).sum())
    pcg_ms = phase_ms["pcg_iterations"]
    slow = float(iters_by_scene.max())
    ent["pcg"] = {"kernel": ("k_pcg_cluster<1..16>" + (" + tile path" if n_tile else "")) if n_tile < len(paths)
                  else "k_spmv + k_update (tile path)",
                  "step_ms": pcg_ms, "algorithmic_bytes_per_step": pcg_bytes, "GB/s": gbs(pcg_bytes, pcg_ms),
                  "frac_hbm": gbs(pcg_bytes, pcg_ms) / peak, "traffic": traffic.get("pcg"),
                  "dram_GB/s": gbs(traffic["pcg"], pcg_ms) if traffic.get("pcg") else None,
                  "dram_frac_hbm": gbs(traffic["pcg"], pcg_ms) / peak if traffic.get("pcg") else None,
                  "scenes_cluster_path": int(len(paths) - n_tile), "scenes_tile_path": n_tile,
                  "iterations_slowest_scene": slow,
                  "us_per_iteration_slowest_scene": 1e3 * pcg_ms / slow if slow else None,
                  "how": "sum over scenes of PCG iterations x (SpMV + update bytes of the scene), over the "
                         "phase's CUDA-event time per step (all refinement sweeps); in a cluster the vectors "
                         "stay in shared memory and the matrix comes from L2 or DRAM, so this is an "
                         "HBM-equivalent rate; traffic and dram_GB/s: the DRAM bytes ncu counts for a step's "
                         "cluster launches (profiles/traffic.json) over the same time"}
    for k in ("spmv", "pcg_update"):
        a = gbs(kbytes[k], kms[k])
        ent[k] = {"kernel": "k_spmv" if k == "spmv" else "k_update", "launch_ms": kms[k],
                  "algorithmic_bytes": kbytes[k], "GB/s": a, "frac_hbm": a / peak, "traffic": traffic.get(k),
                  "note": (f"tile path, timed over every scene of the batch; the step runs it for the {n_tile} "
                           "scene(s) on the tile path only") if n_tile < len(paths) else "tile path (every scene)"}
    if newmark:
        dom = "pcg"
    else:
        dom = max(("element", "assemble", "pcg"), key=lambda k: ent[k]["step_ms"])
    e = ent[dom]
    achieved = e["GB/s"]
    binding = {"element": "FP64 pipe (2 FP64 lanes per SM per clock on GB300): see kernels.element.fp64",
               "assemble": "latency of the gather chains",
               "pcg": "latency: the slowest scene's iterations run one after another (barriers per iteration); "
                      "see kernels.pcg.us_per_iteration_slowest_scene"}[dom]
    return {"kernel": e["kernel"], "phase": dom, "bound": "hbm", "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind, "traffic": e.get("traffic"),
            "algorithmic_bytes": e.get("algorithmic_bytes", e.get("algorithmic_bytes_per_step")),
            "time_ms": e.get("launch_ms", e.get("step_ms")), "binding": binding, "kernels": ent}


def run_ours(args, spec, scene_list):
    import torch
    from hobakv1_gb300 import hobak

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    solver_integrator = {"position": hobak.INTEGRATOR_POSITION, "newmark": hobak.INTEGRATOR_NEWMARK}.get(
        spec.get("integrator"), hobak.INTEGRATOR_VELOCITY)
    opts = hobak.solver_opts(precision=spec["precision"], use_graph=not args.eager, integrator=solver_integrator)
    batch = hobak.BATCH(scene_list, opts)
    if spec.get("contact"):
        ct = spec["contact"]
        for i in range(len(scene_list)):
            batch.set_collisions(i, ct["vf"], ct["eps"], ct["mu"], ct["beta"])
            batch.set_edge_collisions(i, ct["ee"])
    stream = torch.cuda.ExternalStream(batch.stream_handle())
    # launch shapes (tile size, CTA sizes, PCG chunk) from the autotuner, on
    # this batch's data, before the warm-up; the state is left unchanged
    if args.no_autotune and args.cluster_pcg is not None:
        batch.set_tuning(cluster_pcg=args.cluster_pcg)
    if args.no_autotune and args.cluster_max is not None:
        batch.set_tuning(cluster_max=args.cluster_max)
    tuning = batch.get_tuning() if args.no_autotune else batch.autotune(reps=3)

    # ---- device-resident timed region ----
    # (phase timers off: their events split the step graph; the per-phase
    # breakdown is taken after the timed region)
    batch.step(args.warmup)
    # the state the timed steps start from: the e2e loop replays the same steps
    nvs = [s.nv for s in scene_list]
    ntot = 3 * sum(nvs)
    pinned = lambda: torch.empty(ntot, dtype=torch.float64, pin_memory=True).numpy()
    hx, hv, hf = pinned(), pinned(), pinned()
    batch.get_state_all(hx, hv)
    launches0 = batch.launch_count()
    iters = []
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    clocks = ClockSampler(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev[0].record(stream)
    scene_iters = []
    iters_by_scene = np.zeros(len(scene_list))
    for k in range(args.steps):
        st = batch.step(1)
        iters.append(max(s[0] for s in st))
        scene_iters.extend(s[0] for s in st)
        iters_by_scene += [s[0] for s in st]
        ev[k + 1].record(stream)
    torch.cuda.synchronize()
    clock = clocks.stop()
    gpu_launches = batch.launch_count() - launches0
    # per-phase CUDA-event times of a few more steps (outside the timed region)
    phase_steps = min(args.steps, 5)
    batch.enable_timing(True)
    batch.phase_times()  # reset
    batch.step(phase_steps)
    phases = batch.phase_times()
    batch.enable_timing(False)
    iters_by_scene /= max(args.steps, 1)
    lat = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    total_ms = ev[0].elapsed_time(ev[args.steps])
    if world > 1:
        t = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * args.steps / (total_ms / 1e3)

    # ---- rooflines of the kernels the timed step runs ----
    roofline = step_rooflines(batch, spec, scene_list, phases, phase_steps, iters_by_scene, args.workload,
                              clock.get("sm_mhz"))

    # ---- e2e: public API with pinned host buffers in/out every step ----
    # whole-batch calls (every scene's state is contiguous on the device): the
    # inputs x, v, f_ext go up and x, v come back every step; the same steps
    # as the timed region, from the same state (hx, hv saved before it)
    off = 0
    for s in scene_list:
        mass = np.zeros(s.nv)
        np.add.at(mass, s.tets.reshape(-1), np.repeat(0.25 * np.abs(
            np.einsum("ij,ij->i", s.rest[s.tets[:, 3]] - s.rest[s.tets[:, 0]],
                      np.cross(s.rest[s.tets[:, 1]] - s.rest[s.tets[:, 0]],
                               s.rest[s.tets[:, 2]] - s.rest[s.tets[:, 0]])) / 6.0), 4))
        hf[off:off + 3 * s.nv] = (mass[:, None] * (s.density * np.array(s.gravity))[None, :]).reshape(-1)
        off += 3 * s.nv
    e2e_steps = args.steps
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(e2e_steps):
        batch.set_state_all(hx, hv)
        batch.set_external_forces_all(hf)
        batch.step(1)
        batch.get_state_all(hx, hv)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1)
    nbytes = ntot * 8
    e2e = {"value": world * e2e_steps / (e2e_ms / 1e3), "unit": "steps/s",
           "h2d_bytes_per_step": 3 * nbytes, "d2h_bytes_per_step": 2 * nbytes + 136 * len(nvs),
           "api": "hobak_batch_set_state_all/set_external_forces_all/step/get_state_all"}

    # ---- CPU baseline (rank 0, N = 1 only) ----
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        steps = 3 if sum(s.nt for s in scene_list) > 100_000 else 20
        cv, _, cores, sample = cpu_baseline(scene_list, steps, 0, integrator=spec.get("integrator", "velocity"),
                                        contact=spec.get("contact"))
        cpu = {"value": cv, "unit": "steps/s", "cores": cores, "kind": "port",
               "sample": sample + f" of {args.workload} on the host cores (OpenMP), from the initial state",
               "cpu_model": cpu_model(), **port_vs_reference()}

    # the plain FP64 GPU path (one scene at a time) on the same mix, and the
    # same mix batched in FP64 (the precision-only comparison)
    plain = batched64 = None
    if spec["kind"] == "mix" and not args.no_plain and spec["precision"] == 1:
        pv = plain_fp64_gpu(scene_list, 2, integrator=solver_integrator)
        plain = {"value": pv, "unit": "steps/s", "speedup_of_value": value / pv,
                 "how": "each scene its own FP64 batch (CUDA graph per step), scenes stepped one after another"}
        bv, bms, btune = batched_fp64_gpu(scene_list, min(args.steps, 10), args.warmup, solver_integrator,
                                          args.no_autotune)
        batched64 = {"value": bv, "unit": "steps/s", "ms_per_step": bms, "speedup_of_value": value / bv,
                     "launch_shapes": btune,
                     "how": "the same mix as one FP64 batch (CUDA graph per step, autotuned launch shapes), "
                            f"{min(args.steps, 10)} steps after {args.warmup} warm-up steps"}

    if rank == 0:
        lat_sorted = sorted(lat)
        line = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
                "p50_ms": float(np.percentile(lat_sorted, 50)), "p99_ms": float(np.percentile(lat_sorted, 99)),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64" if spec["precision"] == 0 else "f32+f64", "data": "synthetic",
                "config": {"workload": args.workload, **config_of(spec, scene_list)},
                "preconditioner": "block_jacobi",
                "launch_shapes": {**tuning, "chosen_by": "given" if args.no_autotune else "autotuner"},
                "pcg_iters_per_step": float(np.mean(iters)),
                "pcg_iters_per_scene_pct": {q: float(np.percentile(scene_iters, q)) for q in (10, 50, 90, 100)},
                "phases_ms_per_step": {k: v[0] / phase_steps for k, v in phases.items()},
                **({"phases_note": "the Newton loop is one graph node: its element, assembly, rhs and PCG "
                                   "time of every Newton iteration is counted under pcg_iterations"}
                   if spec.get("integrator") == "newmark" else {}),
                "roofline": roofline, "cpu_baseline": cpu, "plain_fp64_gpu": plain, "batched_fp64_gpu": batched64,
                "e2e": e2e,
                "gpu_launches": int(gpu_launches),
                "clocks": clock}
        print(json.dumps(line), flush=True)
    batch.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the unbatched FP64 comparison on mixes")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--serve-impl", default="native", choices=["native", "python"],
                    help="serving workloads: the library's server (hobak_server_*) or the Python one")
    ap.add_argument("--cluster-pcg", type=int, choices=[0, 1], default=None,
                    help="PCG path of the serving cohorts (and of --no-autotune batches): 1 = cluster-resident")
    ap.add_argument("--cluster-max", type=int, choices=[1, 2, 4, 8, 16], default=None,
                    help="largest cluster of --no-autotune batches (the autotuner's choice on the default mix: 8)")
    ap.add_argument("--eager", action="store_true",
                    help="launch kernels one by one instead of the step graph (for per-kernel profilers)")
    args = ap.parse_args()
    spec = WORKLOADS[args.workload]
    scene_list = make_scenes(spec)
    if spec["kind"] == "serve":
        if args.impl == "reference":
            run_reference_serving(args, spec, scene_list)
        elif dist_info()[0] == 0:
            run_serving(args, spec, scene_list)
    elif args.impl == "reference":
        run_reference(args, spec, scene_list)
    else:
        run_ours(args, spec, scene_list)


if __name__ == "__main__":
    main()
