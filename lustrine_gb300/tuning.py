"""Autotuner front end: the launch shape of the PBF iteration kernels (block
size and neighbour gathers in flight per thread) and of the list build,
chosen per GPU and configuration class and cached as JSON.

The timing itself runs in the library (lustrine_pbf_autotune: every
candidate is timed with CUDA events from the same state).  The cache key is
(GPU name, mode, precision, particle-count bucket, solids present, solver
iterations): scenes of the same class share a launch shape.
"""
from __future__ import annotations

import json
import math
import os

from .pbf import PbfSim

CACHE = os.environ.get("LUSTRINE_TUNING_CACHE",
                       os.path.join(os.path.expanduser("~"), ".cache", "lustrine_gb300", "tuning.json"))


def gpu_name() -> str:
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.get_device_name(0)
    except Exception:  # torch is optional for the library
        pass
    return "cuda"


def config_key(sim: PbfSim) -> str:
    p = sim.params
    bucket = int(round(math.log2(max(sim.n, 1))))
    return f"{gpu_name()}|mode{p.mode}|prec{p.precision}|n2^{bucket}|solids{int(sim.ns > 0)}|it{p.iterations}"


def _load(path: str) -> dict:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def tune(sim: PbfSim, dt: float, steps: int = 3, cache: str | None = CACHE, refresh: bool = False) -> dict:
    """Apply the cached launch shape of this configuration class, or run the
    autotuner and cache its choice.  Returns {"tuning": ..., "ms": ..., "cached": bool}."""
    key = config_key(sim)
    db = _load(cache) if cache else {}
    if not refresh and key in db:
        t = db[key]["tuning"]
        sim.set_tuning(t["block"], t["unroll"], t["list_block"], t.get("xsph_unroll", 0),
                       t.get("particles_per_thread", 1), t.get("solver", 0), t.get("solver_threads", 0),
                       t.get("list_format", 1))
        return {"tuning": t, "ms": db[key]["ms"], "cached": True}
    t, ms = sim.autotune(dt, steps)
    if cache:
        db[key] = {"tuning": t, "ms": ms}
        try:
            os.makedirs(os.path.dirname(cache), exist_ok=True)
            tmp = cache + ".tmp"
            with open(tmp, "w") as f:
                json.dump(db, f, indent=1, sort_keys=True)
            os.replace(tmp, cache)
        except OSError:
            pass
    return {"tuning": t, "ms": ms, "cached": False}
