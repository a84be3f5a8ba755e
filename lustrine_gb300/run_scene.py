"""Step one of the benchmark scenes on the GPU and print timing and FP64
statistics.

    python -m lustrine_gb300.run_scene --config config2 --steps 5 [--mixed] [--no-graph]
        [--grid auto|dense|hashed] [--stages] [--shape block,unroll,list_block[,xsph_unroll]] [--sand]

--sand steps the scene's particles with simulate_sand's semantics (sand mode)
instead of the PBF step.

Used for profiling captures of a single configuration (a fixed, short
sequence of launches) and as a quick end-to-end check of an installation.
"""
from __future__ import annotations

import argparse
import json
import time

from . import PRECISION_FP32, PRECISION_MIXED, PbfSim, pbf_params, sand_params, scenes


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="config1", choices=["config0", "config1", "config2", "config4"])
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
    sc = getattr(scenes, a.config)()
    if a.sand:
        p = sand_params(*sc.domain, max_neighbors=max(a.max_neighbors, 96), use_graph=not a.no_graph)
    else:
        p = pbf_params(*sc.domain, iterations=sc.iterations, c_xsph=sc.c_xsph,
                       precision=PRECISION_MIXED if a.mixed else PRECISION_FP32,
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


if __name__ == "__main__":
    raise SystemExit(main())
