"""Step one of the benchmark scenes on the GPU and print timing and FP64
statistics.

    python -m lustrine_gb300.run_scene --config config2 --steps 5 [--mixed | --precision fp32|mixed|scene]
        [--no-graph] [--grid auto|dense|hashed] [--stages] [--shape block,unroll,list_block[,xsph_unroll]]
        [--sand] [--scenes N] [--onchip]

--sand steps the scene's particles with simulate_sand's semantics (sand mode)
instead of the PBF step.  --config config3 steps the first N (--scenes,
default 512) scenes of the batched configuration in one batched context
(--onchip: with the on-chip solve).

Used for profiling captures of a single configuration (a fixed, short
sequence of launches) and as a quick end-to-end check of an installation.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import PRECISION_FP32, PRECISION_MIXED, PRECISION_MIXED_SCENE, PbfSim, pbf_params, sand_params, scenes


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="config1", choices=["config0", "config1", "config2", "config3", "config4"])
    ap.add_argument("--scenes", type=int, default=512, help="config3: scenes in the batch")
    ap.add_argument("--precision", default=None, choices=["fp32", "mixed", "scene"])
    ap.add_argument("--onchip", action="store_true", help="config3: the on-chip solve")
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--mixed", action="store_true")
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--max-neighbors", type=int, default=64)
    ap.add_argument("--grid", default="auto", choices=["auto", "dense", "hashed"])
    ap.add_argument("--stages", action="store_true", help="also print per-stage device ms")
    ap.add_argument("--shape", default=None,
                    help="launch shape block,unroll,list_block[,xsph_unroll] (default: the library's)")
    ap.add_argument("--sand", action="store_true", help="the sand step (simulate_sand semantics)")
    a = ap.parse_args(argv)
    prec = {"fp32": PRECISION_FP32, "mixed": PRECISION_MIXED, "scene": PRECISION_MIXED_SCENE}[
        a.precision or ("mixed" if a.mixed else "fp32")]
    if a.config == "config3":
        return run_batch(a, prec)
    sc = getattr(scenes, a.config)()
    if a.sand:
        p = sand_params(*sc.domain, max_neighbors=max(a.max_neighbors, 96), use_graph=not a.no_graph)
    else:
        p = pbf_params(*sc.domain, iterations=sc.iterations, c_xsph=sc.c_xsph,
                       precision=prec,
                       max_neighbors=a.max_neighbors, use_graph=not a.no_graph,
                       grid_mode=["auto", "dense", "hashed"].index(a.grid))
    with PbfSim(p, sc.n, sc.ns) as sim:
        sim.upload(sc.x, None, sc.solid if sc.ns else None)
        if a.shape:
            sim.set_tuning(*(int(v) for v in a.shape.split(",")))
        t0 = time.perf_counter()
        sim.step(sc.dt, a.steps)
        sim.synchronize()
        wall = time.perf_counter() - t0
        r = sim.reduce()
        out = {"config": sc.name + ("_sand" if a.sand else ""), "n": sc.n, "ns": sc.ns, "steps": a.steps,
               "wall_ms_per_step": wall / max(a.steps, 1) * 1e3, "status": sim.status(),
               "kinetic": r["kinetic"], "com": r["com"], "max_density_error": r["max_density_error"]}
        if a.stages:  # mean of 10 profiled steps
            acc = {}
            for _ in range(10):
                for k, v in sim.profile_step(sc.dt).items():
                    acc[k] = acc.get(k, 0.0) + v[0] / 10
            out["stage_ms"] = {k: round(v, 4) for k, v in acc.items()}
    print(json.dumps(out))
    return 0 if out["status"] == 0 else 1


def run_batch(a, prec):
    scs = scenes.config3(num=a.scenes)
    p = pbf_params(8, 8, 8, iterations=4, precision=prec, max_neighbors=a.max_neighbors,
                   use_graph=not a.no_graph)
    with PbfSim.batch(p, [sc.domain for sc in scs], [sc.n for sc in scs]) as sim:
        if a.onchip:
            sim.set_solver(True)
        sim.upload(np.concatenate([sc.x for sc in scs]))
        if a.shape:
            sim.set_tuning(*(int(v) for v in a.shape.split(",")))
        dt = scs[0].dt
        t0 = time.perf_counter()
        sim.step(dt, a.steps)
        sim.synchronize()
        wall = time.perf_counter() - t0
        r = sim.reduce()
        out = {"config": f"config3_batched_{len(scs)}_scenes", "n": sim.n, "steps": a.steps,
               "solver": sim.solver(), "wall_ms_per_step": wall / max(a.steps, 1) * 1e3, "status": sim.status(),
               "kinetic": r["kinetic"], "max_density_error": r["max_density_error"]}
        if a.stages:
            acc = {}
            for _ in range(10):
                for k, v in sim.profile_step(dt).items():
                    acc[k] = acc.get(k, 0.0) + v[0] / 10
            out["stage_ms"] = {k: round(v, 4) for k, v in acc.items()}
    print(json.dumps(out))
    return 0 if out["status"] == 0 else 1


if __name__ == "__main__":
    raise SystemExit(main())
