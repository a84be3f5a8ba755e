"""Python host side of the GB300 PBF step: a thin object over the lustrine_pbf_*
context API of liblustrine_gb300.so.

    sim = PbfSim(params, n_fluid, n_solid)
    sim.upload(x, v, solid)          # numpy (n, 3) float32 arrays, caller order
    sim.step(dt)                     # CUDA kernels, asynchronous
    x, v = sim.positions(), sim.velocities()

Particle ids: fluid 0..n-1 in the caller's order; solids n..n+ns-1 in the
order given to upload (the reference's storage order of solids).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from ._lib import (MODE_PBF, MODE_REFERENCE, MODE_SAND, PRECISION_FP32, PRECISION_MIXED, PRECISION_MIXED_SCENE,
                   LustrineError,
                   PbfParams, check)

__all__ = ["PbfSim", "PbfParams", "reference_params", "pbf_params", "sand_params", "MODE_PBF",
           "MODE_REFERENCE", "MODE_SAND",
           "PRECISION_FP32", "PRECISION_MIXED", "PRECISION_MIXED_SCENE", "LustrineError"]


def reference_params(X, Y, Z, radius=0.5, kernel_radius_scale=2.0) -> PbfParams:
    """Parameters as init_simulation_extra_parameters sets them
    (Lustrine.cpp:543-555) with the reference's physical defaults
    (Simulation.hpp:147-171), in reference mode."""
    p = PbfParams()
    _lib.load().lustrine_pbf_params_reference(C.byref(p), X, Y, Z, radius, kernel_radius_scale)
    return p


def rest_lattice_mass(rest_density: float, h: float, spacing: float) -> float:
    """The particle mass whose poly6 density (support h) on a cubic lattice
    of the given spacing equals rest_density: rest_density / sum of W over the
    lattice sites closer than h, W(r) = 315 / (64 pi h^9) (h^2 - r^2)^3.  At
    spacing h the neighbours sit where W vanishes and the sum is W(0) alone:
    m = rest_density * 64 pi h^3 / 315 (0.638 at h = 1)."""
    k = int(h // spacing) + 1
    s = 0.0
    for i in range(-k, k + 1):
        for j in range(-k, k + 1):
            for l in range(-k, k + 1):
                r2 = (i * i + j * j + l * l) * spacing * spacing
                if r2 < h * h:
                    s += (h * h - r2) ** 3
    return rest_density / (315.0 / (64.0 * math.pi * h ** 9) * s)


def pbf_params(X, Y, Z, *, radius=0.5, h=1.0, rest_density=1.0, mass=None, gravity=-9.81,
               iterations=4, s_corr_k=0.1, s_corr_n=4.0, s_corr_dq_frac=0.2, c_xsph=0.01,
               epsilon=10.0, precision=PRECISION_FP32, max_neighbors=64, use_graph=True,
               grid_mode=0) -> PbfParams:
    """PBF-mode parameters of the benchmark scenes (dam breaks at unit spacing).

    mass defaults to rest_lattice_mass(rest_density, h, 2 radius): the
    particles' rest lattice is then at the rest density.  A unit mass at rest
    density 1 and h equal to the spacing would put every particle at 1.567
    rest densities on its own, every constraint pushing outwards at rest:
    such a dam break gains energy without bound after about 110 steps."""
    p = reference_params(X, Y, Z, radius, h / radius)
    p.mode = MODE_PBF
    p.precision = precision
    p.rest_density = rest_density
    p.mass = rest_lattice_mass(rest_density, h, 2.0 * radius) if mass is None else mass
    p.gravity[0], p.gravity[1], p.gravity[2] = 0.0, gravity, 0.0
    p.relaxation_epsilon = epsilon
    p.iterations = iterations
    p.s_corr_k = s_corr_k
    p.s_corr_n = s_corr_n
    p.s_corr_dq = s_corr_dq_frac * h
    p.c_xsph = c_xsph
    p.solid_contact = 2.0 * radius
    p.max_neighbors = max_neighbors
    p.use_graph = 1 if use_graph else 0
    p.grid_mode = grid_mode
    return p


def sand_params(X, Y, Z, *, radius=0.5, kernel_radius_scale=2.0, mass=1.0, gravity=-9.81,
                max_neighbors=96, use_graph=True) -> PbfParams:
    """Sand-mode parameters: simulate_sand semantics (Simulate.cpp:156-325)
    on init_simulation_extra_parameters' grid (Lustrine.cpp:543-555)."""
    p = reference_params(X, Y, Z, radius, kernel_radius_scale)
    p.mode = MODE_SAND
    p.mass = mass
    p.gravity[0], p.gravity[1], p.gravity[2] = 0.0, gravity, 0.0
    p.max_neighbors = max_neighbors
    p.use_graph = 1 if use_graph else 0
    return p


def _tuning_dict(t) -> dict:
    return {"block": t.block, "unroll": t.unroll, "list_block": t.list_block, "xsph_unroll": t.xsph_unroll,
            "particles_per_thread": t.particles_per_thread, "solver": t.solver,
            "solver_threads": t.solver_threads, "list_format": t.list_format}


def _f32(a, n):
    a = np.ascontiguousarray(a, dtype=np.float32).reshape(-1)
    if a.size != 3 * n:
        raise ValueError(f"expected {3 * n} floats, got {a.size}")
    return a


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


class PbfSim:
    """One scene on the GPU (a lustrine_pbf context)."""

    def __init__(self, params: PbfParams, n_fluid: int, n_solid: int = 0):
        self.lib = _lib.load()
        self.params = params
        self.n = int(n_fluid)
        self.ns = int(n_solid)
        h = C.c_void_p()
        check(self.lib.lustrine_pbf_create(C.byref(params), self.n, self.ns, C.byref(h)),
              "lustrine_pbf_create")
        self.h = h

    @classmethod
    def batch(cls, params: PbfParams, domains, n_fluid, n_solid=None) -> "PbfSim":
        """Independent scenes stepped together (one launch per stage).
        domains: (S, 3) ints; n_fluid, n_solid: S ints.  Arrays passed to
        upload/download concatenate the scenes in order."""
        self = cls.__new__(cls)
        self.lib = _lib.load()
        self.params = params
        dom = np.ascontiguousarray(domains, np.int32).reshape(-1)
        nf = np.ascontiguousarray(n_fluid, np.int32)
        nsol = None if n_solid is None else np.ascontiguousarray(n_solid, np.int32)
        self.n = int(nf.sum())
        self.ns = 0 if nsol is None else int(nsol.sum())
        self.scene_counts = nf.copy()
        h = C.c_void_p()
        check(self.lib.lustrine_batch_create(C.byref(params), len(nf), _ptr(dom), _ptr(nf), _ptr(nsol),
                                             C.byref(h)), "lustrine_batch_create")
        self.h = h
        return self

    # batches: the on-chip scene solve ----------------------------------------
    def set_solver(self, onchip: bool):
        """The on-chip scene solve (clusters, distributed shared memory) or
        one launch per stage; raises LustrineError (unsupported) where the
        on-chip solve does not apply."""
        check(self.lib.lustrine_batch_set_solver(self.h, 1 if onchip else 0), "batch_set_solver")

    def solver(self) -> str:
        v = C.c_int()
        check(self.lib.lustrine_batch_get_solver(self.h, C.byref(v)), "batch_get_solver")
        return "onchip" if v.value == 1 else "stages"

    def onchip_layout(self) -> dict:
        """Clusters of the on-chip solve's persistent grid, bins of scenes,
        threads per CTA."""
        c, b, t = C.c_int(), C.c_int(), C.c_int()
        check(self.lib.lustrine_batch_onchip_layout(self.h, C.byref(c), C.byref(b), C.byref(t)),
              "batch_onchip_layout")
        return {"clusters": c.value, "bins": b.value, "threads": t.value}

    def set_onchip_threads(self, threads: int):
        check(self.lib.lustrine_batch_set_onchip_threads(self.h, int(threads)), "batch_set_onchip_threads")

    # lifecycle -------------------------------------------------------------
    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.lib.lustrine_pbf_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # state in --------------------------------------------------------------
    def upload(self, x, v=None, solid=None):
        x = _f32(x, self.n)
        v = None if v is None else _f32(v, self.n)
        s = None if (solid is None or self.ns == 0) else _f32(solid, self.ns)
        check(self.lib.lustrine_pbf_upload(self.h, _ptr(x), _ptr(v), _ptr(s)), "upload")

    def upload_device(self, x_ptr: int, v_ptr: int | None, solid_ptr: int | None):
        """Device pointers (e.g. torch tensors' data_ptr()) of 3 floats per particle."""
        check(self.lib.lustrine_pbf_upload_device(self.h, C.c_void_p(x_ptr),
                                                  C.c_void_p(v_ptr) if v_ptr else None,
                                                  C.c_void_p(solid_ptr) if solid_ptr else None),
              "upload_device")

    def upload_state_async(self, x_ptr: int, v_ptr: int | None):
        """Host pointers (page-locked for asynchrony) of x and v, 3 floats each."""
        check(self.lib.lustrine_pbf_upload_state_async(self.h, C.c_void_p(x_ptr),
                                                       C.c_void_p(v_ptr) if v_ptr else None),
              "upload_state_async")

    def set_params(self, params: PbfParams):
        check(self.lib.lustrine_pbf_set_params(self.h, C.byref(params)), "set_params")
        self.params = params

    # stepping --------------------------------------------------------------
    def step(self, dt: float, count: int = 1):
        check(self.lib.lustrine_pbf_steps(self.h, float(dt), int(count)), "step")

    def synchronize(self):
        check(self.lib.lustrine_pbf_synchronize(self.h), "synchronize")

    def stream(self) -> int:
        s = C.c_void_p()
        check(self.lib.lustrine_pbf_stream(self.h, C.byref(s)), "stream")
        return s.value or 0

    def launches_per_step(self) -> int:
        return int(self.lib.lustrine_pbf_launches_per_step(self.h))

    # state out -------------------------------------------------------------
    def download(self, x=True, v=True, lambdas=False, density=False):
        n = self.n
        ax = np.empty((n, 3), np.float32) if x else None
        av = np.empty((n, 3), np.float32) if v else None
        al = np.empty(n, np.float32) if lambdas else None
        ad = np.empty(n, np.float32) if density else None
        check(self.lib.lustrine_pbf_download(self.h, _ptr(ax), _ptr(av), _ptr(al), _ptr(ad)),
              "download")
        return ax, av, al, ad

    def step_host(self, dt: float, x_ptr: int, v_ptr: int | None):
        """Upload x, v from host memory, step, download into them, wait."""
        check(self.lib.lustrine_pbf_step_host(self.h, float(dt), C.c_void_p(x_ptr),
                                              C.c_void_p(v_ptr) if v_ptr else None), "step_host")

    def download_state_async(self, x_ptr: int, v_ptr: int | None):
        check(self.lib.lustrine_pbf_download_state_async(self.h, C.c_void_p(x_ptr),
                                                         C.c_void_p(v_ptr) if v_ptr else None),
              "download_state_async")

    def positions(self):
        return self.download(x=True, v=False)[0]

    def velocities(self):
        return self.download(x=False, v=True)[1]

    def lambdas(self):
        return self.download(x=False, v=False, lambdas=True)[2]

    def density(self):
        return self.download(x=False, v=False, density=True)[3]

    def positions_f64(self):
        out = np.empty((self.n, 3), np.float64)
        check(self.lib.lustrine_pbf_download_positions_f64(self.h, _ptr(out)), "positions_f64")
        return out

    def neighbors(self, cap: int | None = None):
        """(count[n], idx[n, cap]) of the last step, in particle ids."""
        cap = cap or self.params.max_neighbors
        cnt = np.zeros(self.n, np.int32)
        idx = np.full((self.n, cap), -1, np.int32)
        check(self.lib.lustrine_pbf_neighbors(self.h, _ptr(cnt), _ptr(idx), cap), "neighbors")
        return cnt, idx

    def list_format(self) -> str:
        """"compact", "compact_wide" or "column": the form of the last step's
        neighbour lists."""
        v = C.c_int()
        check(self.lib.lustrine_pbf_list_format(self.h, C.byref(v)), "list_format")
        return {_lib.LISTS_COMPACT: "compact", _lib.LISTS_COMPACT_WIDE: "compact_wide"}.get(v.value, "column")

    def reduce(self):
        """FP64 device reductions: mass, momentum[3], kinetic energy,
        centre of mass[3], max |rho/rho0 - 1|."""
        out = (C.c_double * 9)()
        check(self.lib.lustrine_pbf_reduce(self.h, out), "reduce")
        r = list(out)
        return dict(mass=r[0], momentum=r[1:4], kinetic=r[4], com=r[5:8], max_density_error=r[8])

    # launch shape -----------------------------------------------------------
    def get_tuning(self) -> dict:
        t = _lib.PbfTuning()
        check(self.lib.lustrine_pbf_get_tuning(self.h, C.byref(t)), "get_tuning")
        return _tuning_dict(t)

    # sand mode -------------------------------------------------------------
    def set_sand_controls(self, player=None, attract=None, blow=None, attract_radius=None,
                          blow_radius=None, attract_coeff=None, blow_coeff=None, diameter=None):
        """Inputs of the next sand steps (unset arguments keep their value):
        the player's position, the attract and blow flags, their radii and
        coefficients, the contact diameter."""
        c = _lib.SandControls()
        check(self.lib.lustrine_pbf_get_sand_controls(self.h, C.byref(c)), "get_sand_controls")
        if player is not None:
            c.player_position[:] = [float(a) for a in player]
        if attract is not None:
            c.attract_flag = int(bool(attract))
        if blow is not None:
            c.blow_flag = int(bool(blow))
        for name, val in (("attract_radius", attract_radius), ("blow_radius", blow_radius),
                          ("attract_coeff", attract_coeff), ("blow_coeff", blow_coeff),
                          ("particle_diameter", diameter)):
            if val is not None:
                setattr(c, name, float(val))
        check(self.lib.lustrine_pbf_set_sand_controls(self.h, C.byref(c)), "set_sand_controls")

    def attracted(self) -> np.ndarray:
        """Sand mode's per-particle attract flags, current particle order."""
        a = np.zeros(max(self.n, 1), np.int32)
        check(self.lib.lustrine_pbf_get_attracted(self.h, a.ctypes.data), "get_attracted")
        return a[: self.n]

    def set_attracted(self, flags):
        a = np.ascontiguousarray(flags, np.int32).reshape(-1)
        if a.size != self.n:
            raise ValueError(f"expected {self.n} flags, got {a.size}")
        check(self.lib.lustrine_pbf_set_attracted(self.h, a.ctypes.data), "set_attracted")

    def set_tuning(self, block: int, unroll: int, list_block: int, xsph_unroll: int = 0,
                   particles_per_thread: int = 1, solver: int = 0, solver_threads: int = 0,
                   list_format: int = _lib.LISTS_COMPACT):
        """Launch shape (lustrine_pbf_set_tuning); list_format LISTS_COMPACT
        applies where the step allows compact lists, else column lists."""
        t = _lib.PbfTuning(block, unroll, list_block, xsph_unroll, particles_per_thread, solver, solver_threads,
                           list_format)
        check(self.lib.lustrine_pbf_set_tuning(self.h, C.byref(t)), "set_tuning")

    def autotune(self, dt: float, steps: int = 3) -> tuple[dict, float]:
        """Time every launch shape from the current state (state unchanged);
        keeps and returns the fastest with its ms per step."""
        t = _lib.PbfTuning()
        ms = C.c_float()
        check(self.lib.lustrine_pbf_autotune(self.h, float(dt), int(steps), C.byref(t), C.byref(ms)),
              "autotune")
        return _tuning_dict(t), float(ms.value)

    STAGES = ("predict", "scan", "sort", "lists", "lambda", "delta", "xsph", "solve")

    def profile_step(self, dt: float) -> dict:
        """One step with a CUDA event after each stage (direct launches):
        {stage: (milliseconds, events)}."""
        ms = (C.c_double * len(self.STAGES))()
        cnt = (C.c_int * len(self.STAGES))()
        check(self.lib.lustrine_pbf_profile_step(self.h, float(dt), ms, cnt, len(self.STAGES)),
              "profile_step")
        return {k: (ms[i], cnt[i]) for i, k in enumerate(self.STAGES)}

    def reserve(self, capacity: int):
        """Room for up to `capacity` fluid particles (before the first upload)."""
        check(self.lib.lustrine_pbf_reserve(self.h, int(capacity)), "reserve")

    def spawn(self, x, v=None):
        """Append particles (caller indices n, n+1, ...)."""
        x = np.ascontiguousarray(x, np.float32).reshape(-1, 3)
        vv = None if v is None else np.ascontiguousarray(v, np.float32).reshape(-1, 3)
        check(self.lib.lustrine_pbf_spawn(self.h, _ptr(x), _ptr(vv), len(x)), "spawn")
        self.n += len(x)

    def despawn_cells(self, cells) -> int:
        """Remove the particles the last step binned in `cells` (swap-remove
        semantics of the reference's sinks); returns how many left."""
        cells = np.ascontiguousarray(cells, np.int32).reshape(-1)
        out = C.c_int(0)
        check(self.lib.lustrine_pbf_despawn_cells(self.h, _ptr(cells), len(cells), C.byref(out)),
              "despawn_cells")
        self.n -= int(out.value)
        return int(out.value)

    def query_cell_count(self, min_pos, max_pos, include_solid: bool = False) -> int:
        """Particles the last step binned in the cells of the box
        (Lustrine::query_cell_num_particles)."""
        lo = (C.c_float * 3)(*[float(a) for a in min_pos])
        hi = (C.c_float * 3)(*[float(a) for a in max_pos])
        out = C.c_int(0)
        check(self.lib.lustrine_pbf_query_cell_count(self.h, lo, hi, 1 if include_solid else 0,
                                                     C.byref(out)), "query_cell_count")
        return int(out.value)

    def status(self) -> int:
        return int(self.lib.lustrine_pbf_status(self.h))
