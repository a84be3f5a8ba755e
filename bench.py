"""Benchmark of the GB300 PBF step: particle-solver-iterations per second,
batched mixed precision against the plain step, at equal error.

Workload (one line of JSON on rank 0): 512 independent dam-break scenes with
particle counts log-uniform in [1,024, 65,536] (seeded; 7,546,040 particles),
each a jittered block at unit spacing in a box of side 2 ceil(n^(1/3)) and
height ceil(n^(1/3)) + 2, h = 1, 4 solver iterations, dt = 1/60, PBF step
(poly6 / spiky, s_corr, box collision, XSPH).  A "step" is one full step of
every scene (prediction, counting sort, neighbour lists, 4 x (lambda,
delta-p), XSPH and commit).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value     particles x iterations of all scenes / device time per step of the
          batched mixed-precision context (one launch per stage for all
          scenes, the step one CUDA graph; CUDA events on the library's
          stream, max over ranks); L2 flushed (a 256 MiB write) before every
          timed step (the working set, ~1 GB, is larger than L2 anyway).
plain     the plain step on the same scenes: one fp32 context per scene, each
          on its own stream so the scenes' steps overlap; wall clock per step
          of all scenes, and the batched context timed the same way; ratio.
fp64_error  both arms against the FP64 oracle, one step from the same state,
          on the smallest, median and largest scenes: max relative density
          error and max position error (units of h).
e2e       the batched step through the C ABI with the state in page-locked
          host memory (upload x and v, step, download x and v, every step).
roofline  the step's dominant kernel, from a live per-stage CUDA-event
          profile: algorithmic bytes per launch / average launch time; and
          the whole step's algorithmic bytes per particle-iteration.
cpu_baseline  the reference step (the oracle's restatement, one solver
          iteration) over every scene in sequence, scenes spread over all
          host cores (independent scenes; the reference step itself is
          single-threaded).
Multi-GPU (weak scaling): 512 scenes per rank, the 512 N scenes of the same
distribution sharded by scene (longest first to the least-loaded rank); no
collective on the data path.
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
WORKLOAD = "config3_batched_512_scenes"
NUM_SCENES = 512
ITERS = 4

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
# The oracle (oracle/) runs only here: the CPU baseline (the reference step as
# the oracle restates it) and, as the checker, the FP64 step that the GPU
# results are compared with.

def ref_semantics_params(O, domain):
    """Oracle parameters of the reference step (simulate_fluid) on a scene:
    the reference's defaults with the configs' physics."""
    p = O.reference_params(*domain)
    p.rest_density, p.mass, p.relaxation_epsilon = 1.0, 1.0, 10.0
    p.gravity[1] = -9.81
    p.s_corr_dq, p.s_corr_k, p.s_corr_n = 0.2, 0.1, 4.0
    p.clamp_cells = 1
    return p


_WORKER = {}


def _cpu_worker_init(root, num_scenes):
    """Pool worker: the oracle library and the config-3 scenes, built once."""
    if root not in sys.path:
        sys.path.insert(0, root)
    from lustrine_gb300 import scenes
    from oracle import oracle as O
    _WORKER["O"] = O
    _WORKER["scenes"] = scenes.config3(num=num_scenes)


def _cpu_worker_steps(indices):
    """Steps the given scenes once each from their initial state with the
    reference step (one solver iteration); returns (particles, seconds)."""
    O = _WORKER["O"]
    scs = _WORKER["scenes"]
    parts, secs = 0, 0.0
    for i in indices:
        sc = scs[i]
        p = ref_semantics_params(O, sc.domain)
        t0 = time.perf_counter()
        O.compat_step(p, sc.dt, sc.x, np.zeros_like(sc.x))
        secs += time.perf_counter() - t0
        parts += sc.n
    return parts, secs


class CpuScenes:
    """The reference step over config-3 scenes on every host core: a pool of
    worker processes (started with spawn, so it is safe beside a CUDA
    context), each stepping whole scenes (independent units)."""

    def __init__(self, num_scenes, workers=None):
        import multiprocessing as mp
        from oracle import oracle as O
        O.build()  # once, before the workers load it
        self.workers = workers or os.cpu_count() or 1
        self.pool = mp.get_context("spawn").Pool(self.workers, initializer=_cpu_worker_init,
                                                  initargs=(ROOT, num_scenes))

    def step(self, indices, counts):
        """One step of the given scenes, spread over the workers (largest
        scenes first, dealt round-robin); wall seconds and particles."""
        order = sorted(indices, key=lambda i: -counts[i])
        chunks = [order[w::self.workers] for w in range(self.workers)]
        chunks = [c for c in chunks if c]
        t0 = time.perf_counter()
        res = self.pool.map(_cpu_worker_steps, chunks, chunksize=1)
        wall = time.perf_counter() - t0
        return wall, sum(r[0] for r in res)

    def close(self):
        self.pool.close()
        self.pool.join()


def oracle_pbf_params(O, p, domain):
    """Oracle parameters of the PBF step with the GPU context's parameters."""
    q = O.reference_params(*domain, p.particle_radius, p.kernel_radius / p.particle_radius)
    for f in ("rest_density", "mass", "relaxation_epsilon", "s_corr_dq", "s_corr_k", "s_corr_n",
              "c_xsph", "solid_contact", "iterations"):
        setattr(q, f, getattr(p, f))
    for a in range(3):
        q.gravity[a] = p.gravity[a]
    return q


def fp64_errors(p, checks):
    """The checker: the FP64 oracle step from each check's state, and each
    GPU result's max relative density error and max position error against
    it.  checks: [(scene, x0, v0, {arm: (x, rho)})]."""
    from oracle import oracle as O
    O.build()
    out = {}
    for sc, x0, v0, arms in checks:
        q = oracle_pbf_params(O, p, sc.domain)
        o = O.pbf_step(q, sc.dt, x0, v0)
        rho64 = np.asarray(o["density"], np.float64)
        for arm, (x, rho) in arms.items():
            d = out.setdefault(arm, {"max_rel_density_error": 0.0, "max_position_error": 0.0, "scenes": []})
            de = float(np.max(np.abs(np.asarray(rho, np.float64) - rho64) / np.abs(rho64)))
            pe = float(np.max(np.abs(np.asarray(x, np.float64) - o["x"])))
            d["max_rel_density_error"] = max(d["max_rel_density_error"], de)
            d["max_position_error"] = max(d["max_position_error"], pe)
            d["scenes"].append({"particles": sc.n, "rel_density_error": de, "position_error": pe})
    return out


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
    """The reference arm: the reference's fluid step (the oracle's restatement
    of simulate_fluid, bit-exact with the compiled reference; one solver
    iteration) over the same 512 scenes, scenes spread over every host core.
    One step = every scene stepped once from its initial state (a snapshot,
    so every step costs the same)."""
    if rank != 0:
        return
    from lustrine_gb300 import scenes
    counts = [int(c) for c in scenes.batched_counts(NUM_SCENES)]
    cpu = CpuScenes(NUM_SCENES)
    idx = list(range(NUM_SCENES))
    for _ in range(args.warmup):
        cpu.step(idx, counts)
    walls = []
    parts = 0
    for _ in range(args.steps):
        w, parts = cpu.step(idx, counts)
        walls.append(w)
    cpu.close()
    wall = statistics.median(walls)
    value = parts / wall
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded jittered dam-break blocks, log-uniform scene sizes)",
        "config": {"workload": WORKLOAD, "scenes": NUM_SCENES, "fluid_particles": parts,
                   "solver_iterations": 1, "semantics": "reference simulate_fluid, one pass per step",
                   "parallelism": f"{cpu.workers} host processes, whole scenes each"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cpu.workers, "kind": "port",
                         "sample": f"all {NUM_SCENES} scenes per step, median of {args.steps} steps, "
                                   f"each scene from its initial state"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# -------------------------------------------------------------- GPU legs --

def time_steps(sim, dt, steps, flush, ext, launches=None):
    """CUDA-event milliseconds of each of `steps` steps (L2 flushed before
    each); `launches`, a list, receives the library's kernel launches per step.
    The steps run inside the NVTX range "timed" (a profiler can capture them
    alone: ncu --nvtx --nvtx-include timed/)."""
    import torch
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("timed")
    for k in range(steps):
        with torch.cuda.stream(ext):
            flush.zero_()
            starts[k].record(ext)
        sim.step(dt)
        if launches is not None:
            launches.append(sim.launches_per_step())
        with torch.cuda.stream(ext):
            ends[k].record(ext)
    torch.cuda.nvtx.range_pop()
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


def batch_context(scs, precision, dt, warmup):
    """A batched context over the scenes, stepped `warmup` times after the
    autotuner chose its launch shape (timed from that state)."""
    from lustrine_gb300 import PbfSim, pbf_params, tuning
    b = PbfSim.batch(pbf_params(8, 8, 8, iterations=ITERS, precision=precision), [sc.domain for sc in scs],
                     [sc.n for sc in scs])
    b.upload(np.concatenate([sc.x for sc in scs]))
    b.step(dt, 3)
    b.tuned = tuning.tune(b, dt, steps=2, cache=None)
    b.step(dt, warmup)
    b.synchronize()
    return b


def wall_per_step(step_all, steps, flush):
    """Median wall-clock seconds of step_all() with the device synchronised on
    both sides (L2 flushed before each)."""
    import torch
    ts = []
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        step_all()
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    return statistics.median(ts)


def run_ours(args, world, rank, local):
    import torch
    from lustrine_gb300 import PRECISION_MIXED, PRECISION_MIXED_SCENE, PbfSim, pbf_params, scenes, sharding
    torch.cuda.set_device(local)
    allsc = scenes.config3(num=NUM_SCENES * world)
    counts = [sc.n for sc in allsc]
    mine = sharding.my_scenes(counts, world, rank)
    scs = [allsc[i] for i in mine]
    n_local, n_total = sum(sc.n for sc in scs), sum(counts)
    dt = scs[0].dt
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    clocks = ClockSampler()
    clocks.start()  # runs through the warm-up: the timed region is milliseconds long

    b = batch_context(scs, PRECISION_MIXED_SCENE, dt, args.warmup)
    ext = torch.cuda.ExternalStream(b.stream())
    x_keep = torch.empty((n_local, 3), dtype=torch.float32).pin_memory()
    v_keep = torch.empty((n_local, 3), dtype=torch.float32).pin_memory()
    b.download_state_async(x_keep.data_ptr(), v_keep.data_ptr())  # the state the timed region starts from
    b.synchronize()
    barrier(world)
    clocks.mark_start()
    step_launches = []
    ms = time_steps(b, dt, args.steps, flush, ext, step_launches)
    clocks.mark_end()
    status = b.status()
    # keep the GPU on the workload (untimed) while the samples after the timed
    # region arrive
    t_busy = time.time() + 0.5
    while time.time() < t_busy:
        b.step(dt, 5)
        b.synchronize()
    clk = clocks.stop(local, margin=0.5)
    barrier(world)
    ms_step = dist_max(sum(ms) / len(ms), world)
    value = n_total * ITERS / (ms_step * 1e-3)
    launches = int(sum(step_launches))  # the library's kernels in the timed region (no L2 flush)

    # live per-stage profile (CUDA events on the library stream)
    b.upload_state_async(x_keep.data_ptr(), v_keep.data_ptr())
    prof = profile_stages(b, dt)
    peak, peak_kind = measured_peaks()
    cand = {k: v for k, v in prof.items() if k in STAGE_BYTES}
    dom = max(cand, key=lambda k: cand[k][0])
    ms_launch = cand[dom][0] / max(cand[dom][1], 1)
    bytes_launch = STAGE_BYTES[dom] * n_local
    # (under a profiler that serialises the launches the events can read 0)
    achieved = bytes_launch / (ms_launch * 1e-3) / 1e9 if ms_launch > 0 else 0.0
    traffic = read_traffic(dom)
    # whole-step algorithmic bytes per particle-iteration (state traffic model)
    cells = sum((sc.domain[0] + 1) * (sc.domain[1] + 1) * (sc.domain[2] + 1) for sc in scs)
    bpi = 44 + (192 + 8 * cells / n_local) / ITERS
    step_achieved = n_local * ITERS / (ms_step * 1e-3) * bpi / 1e9

    # the plain step on the same scenes: one fp32 context per scene, each on
    # its own stream; both arms timed by wall clock from the same state
    b.upload_state_async(x_keep.data_ptr(), v_keep.data_ptr())
    b.step(dt, 2)
    b.synchronize()
    k_wall = max(3, min(args.steps, 10))
    t_batched = wall_per_step(lambda: b.step(dt), k_wall, flush)
    sims = []
    off = np.concatenate([[0], np.cumsum([sc.n for sc in scs])]).astype(int)
    xs0 = x_keep.numpy()
    vs0 = v_keep.numpy()
    # the per-scene contexts take the batched context's tuned launch shape
    # (the per-stage kernels' shape and list format)
    bt = b.tuned["tuning"]
    plain_shape = dict(block=bt["block"], unroll=bt["unroll"], list_block=bt["list_block"],
                       xsph_unroll=bt["xsph_unroll"], particles_per_thread=bt["particles_per_thread"],
                       list_format=bt.get("list_format", 1))
    for k, sc in enumerate(scs):
        s = PbfSim(pbf_params(*sc.domain, iterations=ITERS), sc.n)
        s.set_tuning(**plain_shape)
        s.upload(xs0[off[k]:off[k + 1]], vs0[off[k]:off[k + 1]])
        s.step(dt, 2)
        sims.append(s)
    torch.cuda.synchronize()

    def step_each():
        for s in sims:
            s.step(dt)

    t_plain = wall_per_step(step_each, k_wall, flush)
    # the other batched arms, from the same state: fp32; mixed with
    # cell-relative iterations; the headline's representation with the
    # on-chip solve
    arms = {}
    b_fp32 = batch_context(scs, 0, dt, 2)
    b_fp32.upload(xs0, vs0)
    b_fp32.step(dt, 2)
    arms["batched_fp32"] = {"wall_ms_per_step": wall_per_step(lambda: b_fp32.step(dt), k_wall, flush) * 1e3,
                            "tuning": b_fp32.tuned["tuning"]}
    b_fp32.close()
    b_rel = batch_context(scs, PRECISION_MIXED, dt, 2)
    b_rel.upload(xs0, vs0)
    b_rel.step(dt, 2)
    arms["batched_mixed_cell_relative"] = {
        "wall_ms_per_step": wall_per_step(lambda: b_rel.step(dt), k_wall, flush) * 1e3,
        "tuning": b_rel.tuned["tuning"]}
    try:
        b.set_solver(True)
        b.upload(xs0, vs0)
        b.step(dt, 2)
        arms["batched_mixed_scene_onchip"] = {"wall_ms_per_step": wall_per_step(lambda: b.step(dt), k_wall,
                                                                                flush) * 1e3,
                                              "layout": b.onchip_layout()}
    except Exception as e:  # the on-chip solve does not apply on this GPU
        arms["batched_mixed_scene_onchip"] = {"unavailable": str(e)}
    b.set_tuning(**b.tuned["tuning"])  # back to the autotuner's choice
    for a in arms.values():
        if "wall_ms_per_step" in a:
            a["over_plain"] = t_plain * 1e3 / a["wall_ms_per_step"]
    # the same two arms along the scenes' 100-step run: the dam breaks
    # compress, the neighbour lists grow (about 4 entries a particle at the
    # start, 9 by step 100) and both arms slow down
    rollout = []
    if not args.no_extras:
        x_init = np.concatenate([sc.x for sc in scs])
        b.upload(x_init, np.zeros_like(x_init))
        done = 0
        for target in (5, 50, 100):
            b.step(dt, target - done)
            done = target
            xt, vt = b.download(x=True, v=True)[:2]
            for k, s in enumerate(sims):
                s.upload(xt[off[k]:off[k + 1]], vt[off[k]:off[k + 1]])
                s.step(dt, 2)
            b.upload(xt, vt)
            b.step(dt, 2)
            torch.cuda.synchronize()
            tb = wall_per_step(lambda: b.step(dt), k_wall, flush)
            tp = wall_per_step(step_each, k_wall, flush)
            b.upload(xt, vt)
            rollout.append({"step": target, "batched_ms_per_step": tb * 1e3, "plain_ms_per_step": tp * 1e3,
                            "batched_over_plain": tp / tb})
    plain = {
        "value": n_local * ITERS / t_plain, "ms_per_step": t_plain * 1e3,
        "contexts": len(sims), "launches_per_step": sum(s.launches_per_step() for s in sims),
        "launch_shape": plain_shape,
        "status": max(s.status() for s in sims), "precision": "fp32",
        "overlap": "one context per scene, each on its own stream: the scenes' steps overlap",
        "batched_mixed_wall_ms_per_step": t_batched * 1e3,
        "batched_mixed_over_plain": t_plain / t_batched,
        "other_batched_arms": arms,
        "rollout": rollout,
        "timing": "wall clock per step of all scenes, device synchronised on both sides, L2 flushed before",
    }

    # one step of both arms from the same state, for the FP64 check below:
    # the smallest, median and largest scenes
    order = np.argsort([sc.n for sc in scs])
    check_ids = [int(order[0]), int(order[len(order) // 2]), int(order[-1])]
    b.upload(xs0, vs0)
    b.step(dt)
    bx, _, _, brho = b.download(x=True, v=False, density=True)
    b_rel.upload(xs0, vs0)
    b_rel.step(dt)
    rx, _, _, rrho = b_rel.download(x=True, v=False, density=True)
    b_rel.close()
    checks = []
    for k in check_ids:
        sims[k].upload(xs0[off[k]:off[k + 1]], vs0[off[k]:off[k + 1]])
        sims[k].step(dt)
        px, _, _, prho = sims[k].download(x=True, v=False, density=True)
        checks.append((scs[k], xs0[off[k]:off[k + 1]].copy(), vs0[off[k]:off[k + 1]].copy(),
                       {"batched_mixed": (bx[off[k]:off[k + 1]], brho[off[k]:off[k + 1]]),
                        "batched_mixed_cell_relative": (rx[off[k]:off[k + 1]], rrho[off[k]:off[k + 1]]),
                        "plain_fp32": (px, prho)}))
    for s in sims:
        s.close()

    # end to end through the C ABI with page-locked host buffers
    e2e = run_e2e_batch(b, x_keep, v_keep, dt, args, world, n_total)
    b.close()

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "impl": "ours",
        "data": "synthetic (seeded jittered dam-break blocks, log-uniform scene sizes)",
        "config": {"workload": WORKLOAD, "scenes": len(allsc), "fluid_particles": n_total,
                   "scene_particles": [int(min(counts)), int(max(counts))], "h": 1.0,
                   "solver_iterations": ITERS, "dt": dt,
                   "precision": "mixed, scene frame (int cell + fp32 offset stored; iterations in fp32 relative "
                                "to each scene's box corner; Kahan density sums; FP64 reductions)",
                   "arm": "batched: one context for all scenes, one CUDA graph per step",
                   "l2": "flushed (256 MiB write) before every timed step; working set ~1 GB > L2",
                   "parallelism": f"scenes sharded over {world} GPU(s)" if world > 1 else "1 GPU",
                   "launch_shape": b.tuned["tuning"]},
        "gpu_launches": launches,
        "status": status,
        "plain": plain,
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
    if rank == 0 and world == 1:
        # the CPU leg: the reference step over the same scenes on every host
        # core, and the FP64 check of both arms
        cpu = CpuScenes(len(allsc))
        walls, parts = [], 0
        for _ in range(2):
            w, parts = cpu.step(mine, counts)
            walls.append(w)
        cpu.close()
        rate = parts / min(walls)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": cpu.workers, "kind": "port",
                                "sample": f"all {len(mine)} scenes stepped once with the reference step "
                                          f"(1 solver iteration), scenes spread over {cpu.workers} host "
                                          f"processes, best of 2 passes ({min(walls):.2f} s)",
                                "nproc": os.cpu_count()}
        line["fp64_error"] = fp64_errors(b.params, checks)
    if not args.no_extras and rank == 0:
        line["variants"] = run_variants(args, flush)
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_e2e_batch(b, x_keep, v_keep, dt, args, world, n_total):
    """The batched step through the C ABI with host buffers: every step
    uploads x and v from page-locked memory, steps all scenes and downloads
    x and v into the same buffers (lustrine_pbf_step_host)."""
    x = x_keep.clone().pin_memory()
    v = v_keep.clone().pin_memory()
    n = x.shape[0]
    steps = max(3, args.steps // 2)
    for _ in range(2):
        b.step_host(dt, x.data_ptr(), v.data_ptr())
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(steps):
        b.step_host(dt, x.data_ptr(), v.data_ptr())
    wall = dist_max((time.perf_counter() - t0) / steps, world)
    return {"value": n_total * ITERS / wall, "unit": UNIT,
            "h2d_bytes_per_step": 2 * 12 * n, "d2h_bytes_per_step": 2 * 12 * n,
            "ms_per_step": wall * 1e3,
            "path": "lustrine_pbf_step_host on the batched context (page-locked host buffers)"}


def run_e2e_scene(sim, sc, args):
    """config 1 through the C ABI with host buffers, and the reference
    wrapper's frame (state on the device, positions to the host every step)."""
    import torch
    n = sc.n
    x = torch.from_numpy(sim.positions()).pin_memory()
    v = torch.from_numpy(sim.velocities()).pin_memory()
    steps = max(3, args.steps // 2)
    for _ in range(2):
        sim.step_host(sc.dt, x.data_ptr(), v.data_ptr())
    t0 = time.perf_counter()
    for _ in range(steps):
        sim.step_host(sc.dt, x.data_ptr(), v.data_ptr())
    dt_wall = (time.perf_counter() - t0) / steps
    return {"value": n * sim.params.iterations / dt_wall, "unit": UNIT,
            "h2d_bytes_per_step": 2 * 12 * n, "d2h_bytes_per_step": 2 * 12 * n,
            "ms_per_step": dt_wall * 1e3,
            "path": "lustrine_pbf_step_host (page-locked host buffers, read and written by the kernels)"}


def run_wrapper_frames(frames):
    """The reference's own C entry points on the global simulation, as a game
    binding calls them: init_grid_box + init_simulation_extra_parameters (a
    64^3 block), set_simulate_function(3) (the PBF step), then per frame
    simulate(dt, false, false) and simulation_bind_positions_copy into
    page-locked host memory.  Wall clock per frame."""
    import torch
    from lustrine_gb300 import wrapper as W
    prm = W.SimulationParameters(128, 72, 128, 0.5, 1.0)
    g = W.init_grid_box(prm, 64, 64, 64, (0.0, 0.0, 0.0))
    W.init_simulation_extra_parameters(prm, [g], [], 1, 2.0, 0)
    st_init = W.last_status()
    W.set_simulate_function(3)
    n = W.get_num_sand_particles()
    buf = torch.empty((n, 3), dtype=torch.float32).pin_memory()
    out = buf.numpy()
    for _ in range(3):
        W.simulate(1.0 / 60.0)
        W.simulation_bind_positions_copy(out)
    ts = []
    for _ in range(frames):
        t0 = time.perf_counter()
        W.simulate(1.0 / 60.0)
        W.simulation_bind_positions_copy(out)
        ts.append(time.perf_counter() - t0)
    st = W.last_status()
    ctx = W.global_context()
    iters = ctx.params.iterations if ctx else 1
    W.cleanup_simulation()
    W.free_grid(g)
    t = statistics.median(ts)
    return {"value": n * iters / t, "unit": UNIT, "ms_per_frame": t * 1e3, "particles": n,
            "solver_iterations": iters, "status": [st_init, st], "d2h_bytes_per_step": 12 * n,
            "path": "simulate + simulation_bind_positions_copy (the reference's wrapper entry points)"}


def run_config1(args, flush):
    """config 1 (262,144 fluid + ~50,000 static particles, PBF): fp32 and
    mixed precision, e2e through the C ABI, the dominant kernel's roofline
    fraction; and the reference semantics on the GPU against the reference
    step on one host core on the same scene (the same work per
    particle-iteration)."""
    from lustrine_gb300 import PRECISION_MIXED, pbf_params, scenes
    k = max(3, min(args.steps, 10))
    sc = scenes.config1()
    out = {}
    for name, prec in (("fp32", 0), ("mixed", PRECISION_MIXED)):
        p = pbf_params(*sc.domain, iterations=sc.iterations, c_xsph=sc.c_xsph, precision=prec)
        sim, _, ms, st = run_scene(sc, p, k, 3, flush)
        prof = profile_stages(sim, sc.dt, reps=2)
        d = prof["delta"]
        ms_l = d[0] / max(d[1], 1)
        out[name] = {"value": sc.n * p.iterations / (np.mean(ms) * 1e-3), "ms_per_step": float(np.mean(ms)),
                     "status": st, "launch_shape": sim.tuned["tuning"],
                     "stage_ms": {a: round(b[0], 4) for a, b in prof.items()},
                     "delta_frac": STAGE_BYTES["delta"] * sc.n / (ms_l * 1e-3) / 1e9 / measured_peaks()[0]}
        if name == "fp32":
            out["e2e"] = run_e2e_scene(sim, sc, args)
        sim.close()
    sem = run_reference_semantics(k, flush)
    rate, nsteps, t = cpu_reference_rate(sc, min(args.cpu_budget, 10.0))
    sem["cpu_port_1_core"] = {"value": rate, "ms_per_step": t * 1e3, "steps": nsteps}
    sem["gpu_over_cpu"] = sem["value"] / rate
    out["reference_semantics"] = sem
    return out


def run_variants(args, flush):
    """Other configurations of the same step (not the headline)."""
    from lustrine_gb300 import PRECISION_MIXED, pbf_params, scenes
    out = {}
    k = max(3, min(args.steps, 10))
    out["config1_voxel_solids_262k"] = run_config1(args, flush)
    sc = scenes.config2()
    p = pbf_params(*sc.domain, iterations=sc.iterations, c_xsph=sc.c_xsph)
    sim, _, ms, st = run_scene(sc, p, k, 3, flush)
    prof = profile_stages(sim, sc.dt, reps=2)
    out["config2_plain_2M"] = {"value": sc.n * p.iterations / (np.mean(ms) * 1e-3),
                               "ms_per_step": float(np.mean(ms)), "status": st,
                               "launch_shape": sim.tuned["tuning"],
                               "stage_ms": {a: round(b[0], 4) for a, b in prof.items()}}
    sim.close()
    out["sand_config1_262k"] = run_sand(k, flush)
    out["sources_sinks_config1"] = run_sources_sinks(max(k, 10))
    out["wrapper_frames_64cube"] = run_wrapper_frames(max(k, 10))
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
                     "constraint_residual_max_abs_rho_over_rho0_minus_1": sim.reduce()["max_density_error"],
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
