"""Python mirror of the reference's C entry points (Lustrine::Wrapper,
src/LustrineWrapper.hpp:86-171) as exported by liblustrine_gb300.so.

The calls keep the reference's names and argument meaning; unlike the
reference, each one's outcome is available from last_status().
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib
from ._lib import Color, GridWrapper, SimulationData, SimulationParameters, Vec3

__all__ = ["SimulationParameters", "SimulationData", "GridWrapper", "Vec3", "Color",
           "query_cell_num_particles", "add_particle_source", "add_particle_sink",
           "set_source_state", "set_sink_state", "get_source_spawned", "get_sink_despawned",
           "init_grid_box", "init_simulation", "init_simulation_extra_parameters", "simulate",
           "simulate_no_flags", "simulation_bind_positions_copy", "cleanup_simulation",
           "get_num_sand_particles", "get_grid_cell_size", "set_simulate_function", "set_player_position",
           "init_grid_magikavoxel", "create_grid", "grid_arrays",
           "last_status", "free_grid"]


def _lib_():
    return _lib.load()


def init_grid_box(params: SimulationParameters, X, Y, Z, position, color=(1, 0, 0, 1), type_=1):
    g = GridWrapper()
    _lib_().init_grid_box(C.byref(params), C.byref(g), X, Y, Z, Vec3(*position), Color(*color), type_)
    return g


def grid_from_cells(cells: np.ndarray, position, type_=0, color=(1, 1, 1, 1)):
    """A GridWrapper over an occupancy array indexed [x, y, z] (the reference's
    grid index x * Y * Z + y * Z + z).  Keep the returned array alive."""
    cells = np.ascontiguousarray(cells, np.int32)
    X, Y, Z = cells.shape
    g = GridWrapper()
    g.cells = cells.ctypes.data_as(C.POINTER(C.c_int))
    g.colors = C.POINTER(Color)()
    g.color = Color(*color)
    g.position = Vec3(*position)
    g.has_one_color_per_cell = False
    g.X, g.Y, g.Z = X, Y, Z
    g.num_grid_cells = X * Y * Z
    g.num_occupied_grid_cells = int((cells != 0).sum())
    g.type = type_
    return g, cells


def init_grid_magikavoxel(path: str, position=(0.0, 0.0, 0.0)) -> GridWrapper:
    """The first model of a MagicaVoxel file as a SOLID grid (cells hold
    colour indices).  Free with free_grid."""
    g = GridWrapper()
    _lib_().init_grid_magikavoxel(C.byref(g), os.fsencode(path), Vec3(*[float(a) for a in position]))
    return g


def create_grid(path: str, type_=0) -> GridWrapper:
    """The same model through the wrapper's create_grid (cells 1, colours in
    double).  Free with free_grid."""
    g = GridWrapper()
    _lib_().create_grid(C.byref(g), str(path), int(type_), len(str(path)))
    return g


def grid_arrays(g: GridWrapper):
    """(cells[X, Y, Z] int32, colors[X, Y, Z, 4] float32) copies of a grid."""
    n = g.X * g.Y * g.Z
    cells = np.ctypeslib.as_array(g.cells, shape=(n,)).copy().reshape(g.X, g.Y, g.Z) if n else np.zeros((0,))
    if g.colors and n:
        colors = np.ctypeslib.as_array(C.cast(g.colors, C.POINTER(C.c_float)), shape=(4 * n,)).copy()
        colors = colors.reshape(g.X, g.Y, g.Z, 4)
    else:
        colors = None
    return cells, colors


def free_grid(g: GridWrapper):
    _lib_().lustrine_free_grid(C.byref(g))


def _grid_array(grids):
    arr = (GridWrapper * max(len(grids), 1))(*grids)
    return arr


def init_simulation(params, sand, solid=(), subdivision=1):
    data = SimulationData()
    sa, so = _grid_array(sand), _grid_array(solid)
    _lib_().init_simulation(C.byref(params), C.byref(data), sa, len(sand), so, len(solid), subdivision)
    return data


def init_simulation_extra_parameters(params, sand, solid=(), subdivision=1, kernel_radius_scale=2.0,
                                     with_credits=0):
    data = SimulationData()
    sa, so = _grid_array(sand), _grid_array(solid)
    _lib_().init_simulation_extra_parameters(C.byref(params), C.byref(data), sa, len(sand), so,
                                             len(solid), subdivision, kernel_radius_scale,
                                             with_credits)
    return data


def simulate(dt, attract=False, blow=False):
    _lib_().simulate(dt, attract, blow)


def simulate_no_flags(dt):
    _lib_().simulate_no_flags(dt)


def simulation_bind_positions_copy(out: np.ndarray | None = None) -> np.ndarray:
    n = get_num_sand_particles()
    if out is None:
        out = np.empty((n, 3), np.float32)
    _lib_().simulation_bind_positions_copy(out.ctypes.data_as(C.POINTER(C.c_float)))
    return out


def cleanup_simulation():
    _lib_().cleanup_simulation()


def get_num_sand_particles() -> int:
    return int(_lib_().get_num_sand_particles())


def get_grid_cell_size() -> int:
    return int(_lib_().get_grid_cell_size())


def query_cell_num_particles(min_pos, max_pos, include_solid: bool = False) -> int:
    return int(_lib_().query_cell_num_particles(Vec3(*min_pos), Vec3(*max_pos), bool(include_solid)))


def add_particle_source(pattern: GridWrapper, direction, freq: float, capacity: int = -1) -> int:
    return int(_lib_().add_particle_source(C.byref(pattern), Vec3(*direction), float(freq), int(capacity)))


def add_particle_sink(min_pos, max_pos, frequency: float) -> int:
    return int(_lib_().add_particle_sink(Vec3(*min_pos), Vec3(*max_pos), float(frequency)))


def set_source_state(index: int, state: bool):
    _lib_().set_source_state(int(index), 1 if state else 0)


def set_sink_state(index: int, state: bool):
    _lib_().set_sink_state(int(index), 1 if state else 0)


def get_source_spawned(index: int) -> int:
    return int(_lib_().get_source_spawned(int(index)))


def get_sink_despawned(index: int) -> int:
    return int(_lib_().get_sink_despawned(int(index)))


def set_simulate_function(index: int):
    """0: simulate_sand (the step after init), 2: the fluid step with the
    reference's semantics, 3: the PBF step."""
    _lib_().set_simulate_function(index)


def set_player_position(position):
    """The player's position for the sand step's attract and blow."""
    _lib_().lustrine_set_player_position(Vec3(*[float(a) for a in position]))


def last_status() -> int:
    return int(_lib_().lustrine_last_status())


def global_context():
    """The lustrine_pbf context behind the wrapper simulation (a PbfSim view)."""
    from .pbf import PbfSim
    h = _lib_().lustrine_global_context()
    if not h:
        return None
    sim = PbfSim.__new__(PbfSim)
    sim.lib = _lib_()
    sim.h = C.c_void_p(h)
    n, ns = C.c_int(), C.c_int()
    _lib_().lustrine_pbf_counts(sim.h, C.byref(n), C.byref(ns))
    sim.n, sim.ns = n.value, ns.value
    p = _lib.PbfParams()
    _lib_().lustrine_pbf_get_params(sim.h, C.byref(p))
    sim.params = p
    sim.close = lambda: None  # owned by the wrapper singleton
    return sim
