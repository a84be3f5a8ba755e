"""Benchmark of the GB300 PBF step: particle-solver-iterations per second.

Workload (one line of JSON on rank 0): the voxel-solid dam break -- 262,144
fluid particles (64^3 jittered lattice) and ~50k static solid particles from
a seeded 64 x 64 heightmap in a 128 x 64 x 128 box, h = 1, 4 solver
iterations, dt = 1/60, PBF step (poly6 / spiky, s_corr, box and solid
collision, XSPH).  A "step" is one full step (prediction, counting sort,
neighbour lists, 4 x (lambda, delta-p), XSPH and commit).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value     sum over ranks of fluid particles x iterations / device time per
          step (CUDA events on the library's stream, max over ranks); L2 is
          flushed (a 256 MiB write) before every timed step.
e2e       the same metric through the C ABI with the state in page-locked
          host memory: every step uploads x and v, steps, downloads x and v.
roofline  the step's dominant kernel, from a live per-stage CUDA-event
          profile: algorithmic bytes per launch / average launch time.
cpu_baseline  the oracle's restatement of the reference step (one solver
          iteration, single thread) on the same scene, on this host.
Multi-GPU: every rank steps its own replica (the scene does not shard; no
collective on the data path), scaling "weak".
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "PBF particle-solver-iters/s"
UNIT = "particle-iters/s"
WORKLOAD = "config1_voxel_solids_262k"

# Algorithmic bytes per particle per launch of each stage: compulsory fp32
# state traffic (positions 12 B, lambda 4 B; neighbour gathers counted as
# cache hits).
STAGE_BYTES = {"lambda": 12 + 4, "delta": 12 + 4 + 12}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=20.0, help="seconds of CPU baseline work")
    return ap.parse_args()


# ------------------------------------------------------------------ helpers --

def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock and throttle-reason samples (every 200 ms), each
    stamped with the host time it arrived.  A timed region of a few
    milliseconds falls between two samples, so the sampler runs from before
    the warm-up (the GPU under the same load) and stop() keeps the samples
    within `margin` seconds of the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.lines = []
        self.t0 = self.t1 = None

    def start(self):
        import threading
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return

        def pump():
            for line in self.proc.stdout:
                self.lines.append((time.time(), line))

        self.thread = threading.Thread(target=pump, daemon=True)
        self.thread.start()
        # wait (up to 5 s) for the first sample so the timed region is covered
        t_end = time.time() + 5.0
        while not self.lines and time.time() < t_end and self.proc.poll() is None:
            time.sleep(0.02)

    def mark_start(self):
        self.t0 = time.time()

    def mark_end(self):
        self.t1 = time.time()

    def stop(self, gpu_index=0, margin=1.0):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(2)
        lo = (self.t0 or 0.0) - margin
        hi = (self.t1 or time.time()) + margin
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for t, line in self.lines:
            if not lo <= t <= hi:
                continue
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9 or not parts[0].isdigit() or int(parts[0]) != gpu_index:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        region = (self.t1 - self.t0) if (self.t0 and self.t1) else None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm), "window": f"timed region ({region:.3f} s) +- {margin} s, "
                                              f"GPU stepping the workload throughout"
                if region is not None else "whole run"}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        if args.impl == "ours":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def dist_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# --------------------------------------------------------------- CPU legs --

def cpu_reference_rate(scene, budget_s, min_steps=3):
    """The reference step restated by the oracle (one solver iteration, single
    thread): median time of steps each restored from the same snapshot."""
    from oracle import oracle as O
    O.build()
    p = O.reference_params(*scene.domain)
    p.rest_density, p.mass, p.relaxation_epsilon = 1.0, 1.0, 10.0
    p.gravity[1] = -9.81
    p.s_corr_dq, p.s_corr_k, p.s_corr_n = 0.2, 0.1, 4.0
    p.clamp_cells = 1
    v0 = np.zeros_like(scene.x)
    times = []
    t_start = time.perf_counter()
    while len(times) < min_steps or (time.perf_counter() - t_start < budget_s and len(times) < 50):
        t0 = time.perf_counter()
        O.compat_step(p, scene.dt, scene.x, v0, solid=scene.solid if scene.ns else None)
        times.append(time.perf_counter() - t0)
        if time.perf_counter() - t_start > 3 * budget_s:
            break
    t = statistics.median(times)
    return scene.n / t, len(times), t


def cpu_sand_rate(scene, x, v, reps=3):
    """The reference's sand step restated by the oracle (single thread) on the
    given state: median time of `reps` steps from it.  Particle-substeps/s."""
    from oracle import oracle as O
    O.build()
    p = O.reference_params(*scene.domain)
    p.mass = 1.0
    p.gravity[1] = -9.81
    ctl = O.sand_controls(diameter=1.0)
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        O.sand_step(p, ctl, np.float32(scene.dt), x, v, None, solid=scene.solid, cap=96)
        times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    return scene.n * 4 / t, t


def run_reference(args, world, rank):
    if rank != 0:
        return
    from lustrine_gb300 import scenes
    sc = scenes.config1()
    rates = []
    for _ in range(args.warmup):
        cpu_reference_rate(sc, 0.0, min_steps=1)
    for _ in range(args.steps):
        r, _, _ = cpu_reference_rate(sc, 0.0, min_steps=1)
        rates.append(r)
    value = statistics.median(rates)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": sc.n / value * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded jittered lattice + seeded heightmap solids)",
        "config": {"workload": WORKLOAD, "fluid_particles": sc.n, "solid_particles": sc.ns,
                   "solver_iterations": 1, "semantics": "reference simulate_fluid, one pass"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": f"{args.steps} single steps of the full scene from one snapshot"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# -------------------------------------------------------------- GPU legs --

def time_steps(sim, dt, steps, flush, ext, launches=None):
    """CUDA-event milliseconds of each of `steps` steps (L2 flushed before
    each); `launches`, a list, receives the library's kernel launches per step."""
    import torch
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    torch.cuda.synchronize()
    for k in range(steps):
        with torch.cuda.stream(ext):
            flush.zero_()
            starts[k].record(ext)
        sim.step(dt)
        if launches is not None:
            launches.append(sim.launches_per_step())
        with torch.cuda.stream(ext):
            ends[k].record(ext)
    torch.cuda.synchronize()
    return [s.elapsed_time(e) for s, e in zip(starts, ends)]


def profile_stages(sim, dt, reps=3):
    acc = {}
    for _ in range(reps):
        for k, (ms, cnt) in sim.profile_step(dt).items():
            a = acc.setdefault(k, [0.0, 0])
            a[0] += ms / reps
            a[1] = cnt
    return acc


def run_scene(sc, params, steps, warmup, flush):
    import torch
    from lustrine_gb300 import PbfSim, tuning
    sim = PbfSim(params, sc.n, sc.ns)
    sim.upload(sc.x, None, sc.solid if sc.ns else None)
    sim.step(sc.dt, warmup)
    sim.synchronize()
    # launch shape chosen by the autotuner on this GPU (timed from this state)
    sim.tuned = tuning.tune(sim, sc.dt, steps=3, cache=None)
    ext = torch.cuda.ExternalStream(sim.stream())
    ms = time_steps(sim, sc.dt, steps, flush, ext)
    st = sim.status()
    return sim, ext, ms, st


def run_ours(args, world, rank, local):
    import torch
    from lustrine_gb300 import PRECISION_MIXED, pbf_params, scenes
    torch.cuda.set_device(local)
    sc = scenes.config1()
    params = pbf_params(*sc.domain, iterations=sc.iterations, c_xsph=sc.c_xsph)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    clocks = ClockSampler()
    clocks.start()  # runs through the warm-up: the timed region is milliseconds long

    sim, ext, _, _ = run_scene(sc, params, 1, args.warmup, flush)  # warm-up, graph capture
    barrier(world)
    clocks.mark_start()
    step_launches = []
    ms = time_steps(sim, sc.dt, args.steps, flush, ext, step_launches)
    clocks.mark_end()
    status = sim.status()
    # keep the GPU on the workload (untimed) while the samples after the
    # timed region arrive, then put back the state the timed region left (the
    # thousands of extra steps would carry the scene far from it)
    keep_x = torch.empty((sc.n, 3), dtype=torch.float32).pin_memory()
    keep_v = torch.empty((sc.n, 3), dtype=torch.float32).pin_memory()
    sim.download_state_async(keep_x.data_ptr(), keep_v.data_ptr())
    sim.synchronize()
    t_busy = time.time() + 0.5
    while time.time() < t_busy:
        sim.step(sc.dt, 20)
        sim.synchronize()
    clk = clocks.stop(local, margin=0.5)
    sim.upload_state_async(keep_x.data_ptr(), keep_v.data_ptr())
    sim.synchronize()
    barrier(world)
    ms_step = dist_max(sum(ms) / len(ms), world)
    iters = params.iterations
    value = world * sc.n * iters / (ms_step * 1e-3)
    launches = int(sum(step_launches))  # the library's kernels in the timed region (no L2 flush)

    # live per-stage profile (CUDA events on the library stream)
    prof = profile_stages(sim, sc.dt)
    peak, peak_kind = measured_peaks()
    cand = {k: v for k, v in prof.items() if k in STAGE_BYTES}
    dom = max(cand, key=lambda k: cand[k][0])
    ms_launch = cand[dom][0] / max(cand[dom][1], 1)
    bytes_launch = STAGE_BYTES[dom] * sc.n
    achieved = bytes_launch / (ms_launch * 1e-3) / 1e9
    traffic = read_traffic(dom)
    # whole-step algorithmic bytes per particle-iteration (state traffic model)
    cells = (sc.domain[0] + 1) * (sc.domain[1] + 1) * (sc.domain[2] + 1)
    bpi = 44 + (192 + 8 * cells / sc.n + 12 * sc.ns / sc.n) / iters
    step_achieved = value / world * bpi / 1e9

    # end to end through the C ABI with page-locked host buffers
    e2e = run_e2e(sim, sc, args, ext)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "impl": "ours",
        "data": "synthetic (seeded jittered lattice + seeded heightmap solids)",
        "config": {"workload": WORKLOAD, "fluid_particles": sc.n, "solid_particles": sc.ns,
                   "box": list(sc.domain), "h": 1.0, "solver_iterations": iters, "dt": sc.dt,
                   "precision": "fp32", "l2": "flushed (256 MiB write) before every timed step",
                   "parallelism": f"replicas x{world}", "launch_shape": sim.tuned["tuning"]},
        "gpu_launches": launches,
        "status": status,
        "e2e": e2e,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": traffic, "bytes_per_launch": bytes_launch,
                     "ms_per_launch": ms_launch},
        "step_roofline": {"bytes_per_particle_iter": bpi, "achieved": step_achieved,
                          "frac": step_achieved / peak, "unit": "GB/s"},
        "stage_ms": {k: round(v[0], 5) for k, v in prof.items()},
    }
    if clk:
        line["clocks"] = clk
    if rank == 0:
        rate, nsteps, t = cpu_reference_rate(sc, args.cpu_budget)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": f"median of {nsteps} single reference-semantics steps "
                                          f"(1 solver iteration) of the full scene from one "
                                          f"snapshot, {t * 1e3:.1f} ms each",
                                "nproc": os.cpu_count()}
    if not args.no_extras and rank == 0:
        line["variants"] = run_variants(args, flush)
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_e2e(sim, sc, args, ext):
    import torch
    n = sc.n
    x = torch.from_numpy(sim.positions()).pin_memory()
    v = torch.from_numpy(sim.velocities()).pin_memory()
    steps = max(3, args.steps // 2)
    for _ in range(2):
        sim.step_host(sc.dt, x.data_ptr(), v.data_ptr())
    t0 = time.perf_counter()
    for _ in range(steps):
        # uploads x, v, steps, downloads x, v into the same page-locked
        # buffers and waits: the host holds the step's result
        sim.step_host(sc.dt, x.data_ptr(), v.data_ptr())
    dt_wall = (time.perf_counter() - t0) / steps
    # the reference wrapper's frame (simulate, then simulation_bind_positions_copy):
    # the state stays on the device, the positions come to the host every step
    sim.synchronize()
    for _ in range(2):
        sim.step(sc.dt)
        sim.download_state_async(x.data_ptr(), None)
        sim.synchronize()
    t1 = time.perf_counter()
    for _ in range(steps):
        sim.step(sc.dt)
        sim.download_state_async(x.data_ptr(), None)
        sim.synchronize()
    frame = (time.perf_counter() - t1) / steps
    return {"value": n * sim.params.iterations / dt_wall, "unit": UNIT,
            "h2d_bytes_per_step": 2 * 12 * n, "d2h_bytes_per_step": 2 * 12 * n,
            "ms_per_step": dt_wall * 1e3,
            "path": "lustrine_pbf_step_host (page-locked host buffers, read and written by the kernels)",
            "positions_out_frame": {"value": n * sim.params.iterations / frame, "ms_per_step": frame * 1e3,
                                    "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 12 * n,
                                    "path": "state resident on the device, positions to page-locked host "
                                            "memory every step (the reference wrapper's simulate + "
                                            "simulation_bind_positions_copy frame)"}}


def run_variants(args, flush):
    """Other configurations of the same step (not the headline)."""
    from lustrine_gb300 import PRECISION_MIXED, pbf_params, scenes
    out = {}
    k = max(3, min(args.steps, 10))
    sc = scenes.config1()
    p = pbf_params(*sc.domain, iterations=sc.iterations, c_xsph=sc.c_xsph, precision=PRECISION_MIXED)
    sim, _, ms, st = run_scene(sc, p, k, 3, flush)
    out["config1_mixed"] = {"value": sc.n * p.iterations / (np.mean(ms) * 1e-3),
                            "ms_per_step": float(np.mean(ms)), "status": st,
                            "launch_shape": sim.tuned["tuning"]}
    sim.close()
    # the same step without programmatic dependent launch between kernels
    os.environ["LUSTRINE_NO_PDL"] = "1"
    p = pbf_params(*sc.domain, iterations=sc.iterations, c_xsph=sc.c_xsph)
    sim, _, ms, st = run_scene(sc, p, k, 3, flush)
    del os.environ["LUSTRINE_NO_PDL"]
    out["config1_no_pdl"] = {"value": sc.n * p.iterations / (np.mean(ms) * 1e-3),
                             "ms_per_step": float(np.mean(ms)), "status": st}
    sim.close()
    sc = scenes.config2()
    p = pbf_params(*sc.domain, iterations=sc.iterations, c_xsph=sc.c_xsph)
    sim, _, ms, st = run_scene(sc, p, k, 3, flush)
    prof = profile_stages(sim, sc.dt, reps=2)
    out["config2_plain_2M"] = {"value": sc.n * p.iterations / (np.mean(ms) * 1e-3),
                               "ms_per_step": float(np.mean(ms)), "status": st,
                               "launch_shape": sim.tuned["tuning"],
                               "stage_ms": {a: round(b[0], 4) for a, b in prof.items()}}
    sim.close()
    out["reference_semantics_config1"] = run_reference_semantics(k, flush)
    out["sand_config1_262k"] = run_sand(k, flush)
    out["sources_sinks_config1"] = run_sources_sinks(max(k, 10))
    out["config3_batched_vs_plain"] = run_config3(max(3, min(args.steps, 10)), flush)
    # 4,194,304 particles in a 4096 x 256 x 4096 box: 4.3e9 cells, so the
    # grid is hashed (2^23 buckets); mixed precision is the mode the box needs
    sc = scenes.config4()
    for name, prec in (("config4_mixed_hashed_4M", PRECISION_MIXED), ("config4_fp32_hashed_4M", 0)):
        p = pbf_params(*sc.domain, iterations=sc.iterations, c_xsph=sc.c_xsph, precision=prec)
        sim, _, ms, st = run_scene(sc, p, k, 3, flush)
        prof = profile_stages(sim, sc.dt, reps=2)
        out[name] = {"value": sc.n * p.iterations / (np.mean(ms) * 1e-3),
                     "ms_per_step": float(np.mean(ms)), "status": st,
                     "launch_shape": sim.tuned["tuning"],
                     "max_density_error": sim.reduce()["max_density_error"],
                     "stage_ms": {a: round(b[0], 4) for a, b in prof.items()}}
        sim.close()
    return out


def run_reference_semantics(steps, flush):
    """The reference's fluid step semantics on the GPU (mode R: one lambda
    and one position pass, cubic kernel, Jacobi update) on config 1's scene:
    the same work per particle-iteration as the CPU reference arm."""
    import torch
    from lustrine_gb300 import PbfSim, reference_params, scenes
    sc = scenes.config1()
    p = reference_params(*sc.domain)
    p.rest_density, p.mass, p.relaxation_epsilon = 1.0, 1.0, 10.0
    p.gravity[1] = -9.81
    p.s_corr_dq, p.s_corr_k, p.s_corr_n = 0.2, 0.1, 4.0
    p.clamp_cells = 1
    sim = PbfSim(p, sc.n, sc.ns)
    sim.upload(sc.x, None, sc.solid)
    sim.step(sc.dt, 3)
    sim.synchronize()
    ext = torch.cuda.ExternalStream(sim.stream())
    ms = time_steps(sim, sc.dt, steps, flush, ext)
    out = {"value": sc.n / (np.median(ms) * 1e-3), "unit": UNIT, "ms_per_step": float(np.median(ms)),
           "status": sim.status(), "launches_per_step": sim.launches_per_step(), "solver_iterations": 1}
    sim.close()
    return out


def run_sand(steps, flush):
    """simulate_sand on the GPU (sand mode: integration, stable cell sort,
    symmetric lists, 4 contact/friction substeps) on config 1's scene with the
    64^3 block as sand over the heightmap's static particles.  Rate in
    particle-substeps/s from CUDA-event step times (L2 flushed before each),
    and the oracle's restatement of the reference's sand step timed on one
    host core from the same state."""
    import torch
    from lustrine_gb300 import PbfSim, sand_params, scenes
    sc = scenes.config1()
    sim = PbfSim(sand_params(*sc.domain), sc.n, sc.ns)
    sim.upload(sc.x, None, sc.solid)
    sim.step(sc.dt, 5)
    sim.synchronize()
    ext = torch.cuda.ExternalStream(sim.stream())
    ms = time_steps(sim, sc.dt, steps, flush, ext)
    prof = profile_stages(sim, sc.dt, reps=2)
    x, v, _, _ = sim.download()
    out = {"value": sc.n * 4 / (np.median(ms) * 1e-3), "unit": "particle-substeps/s",
           "ms_per_step": float(np.median(ms)), "status": sim.status(),
           "launches_per_step": sim.launches_per_step(), "sand_particles": sc.n, "static_particles": sc.ns,
           "stage_ms": {a: round(b[0], 4) for a, b in prof.items() if b[1]}}
    sim.close()
    rate, t = cpu_sand_rate(sc, x, v)
    out["cpu_baseline"] = {"value": rate, "unit": "particle-substeps/s", "cores": 1, "kind": "port",
                           "ms_per_step": t * 1e3,
                           "sample": "median of 3 single steps of the full scene from the GPU's state"}
    return out


def run_sources_sinks(frames):
    """Particles entering and leaving config 1's scene on the device: each
    frame spawns a 16 x 16 sheet of particles (a source), steps, and removes
    the particles binned in 16 x 16 floor cells (a sink, the reference's
    swap-remove order); the count the sink returns ends each frame on the
    host.  Wall-clock milliseconds per frame against the same frames without
    source and sink, and the cell-count query (Lustrine::query_cell_num_particles)
    over the whole box and over a 16^3 region, per call."""
    from lustrine_gb300 import PbfSim, pbf_params, scenes
    sc = scenes.config1()
    p = pbf_params(*sc.domain, iterations=sc.iterations, c_xsph=sc.c_xsph)
    sheet = scenes.lattice((16, 1, 16), (104, 40, 40))
    gx, gz = sc.domain[0] + 1, sc.domain[2] + 1
    # floor cells beside the block (x 20-35, z 64-79), where the dam break spreads
    sink = np.array([0 * gx * gz + x * gz + z for x in range(20, 36) for z in range(64, 80)], np.int32)
    out = {"spawned_per_frame": len(sheet), "sink_cells": len(sink), "frames": frames}
    for name, dynamic in (("plain", False), ("sources_sinks", True)):
        sim = PbfSim(p, sc.n, sc.ns)
        sim.reserve(sc.n + len(sheet) * (frames + 5))
        sim.upload(sc.x, None, sc.solid)
        sim.step(sc.dt, 3)
        sim.synchronize()
        ts, removed = [], 0
        for _ in range(frames):
            t0 = time.perf_counter()
            if dynamic:
                sim.spawn(sheet)
            sim.step(sc.dt)
            if dynamic:
                removed += sim.despawn_cells(sink)
            else:
                sim.synchronize()
            ts.append(time.perf_counter() - t0)
        out[name + "_ms_per_frame"] = float(np.median(ts) * 1e3)
        if dynamic:
            out["removed_total"] = removed
            out["particles_after"] = sim.n
            out["status"] = sim.status()
            for label, lo, hi in (("query_whole_box_us", (0, 0, 0), sc.domain),
                                  ("query_16cube_us", (40, 8, 40), (56, 24, 56))):
                q = []
                for _ in range(20):
                    t0 = time.perf_counter()
                    sim.query_cell_count(lo, hi)
                    q.append(time.perf_counter() - t0)
                out[label] = float(np.median(q) * 1e6)
        sim.close()
    return out


def run_config3(steps, flush):
    """512 independent scenes (log-uniform 1,024-65,536 particles): the batched
    step (one launch per stage for all scenes, fp32 and mixed precision)
    against the plain step applied scene by scene (one context and stream per
    scene), both with the scenes' steps overlapping on the GPU and one after
    another.  Wall-clock time per step of all scenes, device synchronised,
    L2 flushed before each step; the equal-error condition (batched mixed
    density within 1e-4 of FP64) is asserted by tests/test_gpu_batch.py."""
    import torch
    from lustrine_gb300 import PRECISION_MIXED, PbfSim, pbf_params, scenes, tuning
    scs = scenes.config3()
    total = sum(sc.n for sc in scs)
    dt = scs[0].dt
    x_all = np.concatenate([sc.x for sc in scs])
    out = {"scenes": len(scs), "fluid_particles": total, "iterations": 4}

    def wall(step_all):
        ts = []
        for _ in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            step_all()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        return statistics.median(ts)

    for name, prec in (("batched_fp32", 0), ("batched_mixed", PRECISION_MIXED)):
        b = PbfSim.batch(pbf_params(8, 8, 8, iterations=4, precision=prec), [sc.domain for sc in scs],
                         [sc.n for sc in scs])
        b.upload(x_all)
        b.step(dt, 3)
        tuned = tuning.tune(b, dt, steps=2, cache=None)
        b.step(dt, 2)
        t = wall(lambda: b.step(dt))
        out[name] = {"value": total * 4 / t, "ms_per_step": t * 1e3, "status": b.status(),
                     "launch_shape": tuned["tuning"], "launches_per_step": b.launches_per_step()}
        b.close()
    sims = []
    for sc in scs:
        s = PbfSim(pbf_params(*sc.domain, iterations=4), sc.n)
        s.upload(sc.x)
        s.step(dt, 2)
        sims.append(s)

    def step_each():
        for s in sims:
            s.step(dt)

    t = wall(step_each)
    out["plain_per_scene"] = {"value": total * 4 / t, "ms_per_step": t * 1e3,
                              "status": max(s.status() for s in sims),
                              "launches_per_step": sum(s.launches_per_step() for s in sims),
                              "overlap": "each scene's context on its own stream: the scenes' steps overlap"}

    def step_each_serial():
        for s in sims:
            s.step(dt)
            s.synchronize()

    t = wall(step_each_serial)
    out["plain_serial"] = {"value": total * 4 / t, "ms_per_step": t * 1e3,
                           "status": max(s.status() for s in sims),
                           "overlap": "none: each scene's step completes before the next is issued"}
    for s in sims:
        s.close()
    out["batched_mixed_over_plain"] = out["batched_mixed"]["value"] / out["plain_per_scene"]["value"]
    out["batched_mixed_over_plain_serial"] = out["batched_mixed"]["value"] / out["plain_serial"]["value"]
    return out


def read_traffic(kernel):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary (profiles/), or None."""
    path = os.path.join(ROOT, "profiles", f"ncu_{kernel}_{WORKLOAD}.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("traffic_bytes_per_launch:"):
            return float(line.split(":", 1)[1])
    return None


def main():
    args = parse()
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
