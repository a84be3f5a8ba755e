"""ctypes binding of liblustrine_gb300.so (the C ABI in include/lustrine_gb300.h).

The library is the product: every call below goes to CUDA kernels.  There is
no CPU fallback -- if the library is missing and cannot be built, importing
the binding raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

LUSTRINE_OK = 0
ERRORS = {
    1: "LUSTRINE_ERR_ARGS",
    2: "LUSTRINE_ERR_CUDA",
    3: "LUSTRINE_ERR_NOMEM",
    4: "LUSTRINE_ERR_NBR_OVERFLOW",
    5: "LUSTRINE_ERR_CELL_RANGE",
    6: "LUSTRINE_ERR_UNSUPPORTED",
    7: "LUSTRINE_ERR_NO_SIMULATION",
    8: "LUSTRINE_ERR_TIMEOUT",
    9: "LUSTRINE_ERR_BAD_VALUE",
    10: "LUSTRINE_ERR_TOO_LARGE",
}
MODE_REFERENCE, MODE_PBF, MODE_SAND = 0, 1, 2
SOLVER_STAGES, SOLVER_ONCHIP = 0, 1
PRECISION_FP32, PRECISION_MIXED, PRECISION_MIXED_SCENE = 0, 1, 2


class LustrineError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        self.code = code
        super().__init__(f"{what}: {ERRORS.get(code, code)}" if what else ERRORS.get(code, str(code)))


# ------------------------------------------------------------ C structures --

class SimulationParameters(C.Structure):
    _fields_ = [("X", C.c_int), ("Y", C.c_int), ("Z", C.c_int),
                ("particleRadius", C.c_float), ("particleDiameter", C.c_float)]


class SimulationData(C.Structure):
    _fields_ = [("num_sand_particles", C.c_int), ("num_solid_particles", C.c_int),
                ("start_sand_index", C.c_int), ("end_sand_index", C.c_int),
                ("start_solid_index", C.c_int), ("end_solid_index", C.c_int)]


class Color(C.Structure):
    _fields_ = [("r", C.c_float), ("g", C.c_float), ("b", C.c_float), ("a", C.c_float)]


class Vec3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class GridWrapper(C.Structure):
    _fields_ = [("cells", C.POINTER(C.c_int)), ("colors", C.POINTER(Color)), ("color", Color),
                ("position", Vec3), ("has_one_color_per_cell", C.c_bool), ("X", C.c_int),
                ("Y", C.c_int), ("Z", C.c_int), ("num_grid_cells", C.c_int),
                ("num_occupied_grid_cells", C.c_int), ("type", C.c_int)]


class BindingString(C.Structure):
    _fields_ = [("length", C.c_int64), ("data", C.c_char_p)]


class PbfParams(C.Structure):
    _fields_ = [("mode", C.c_int), ("precision", C.c_int), ("domain", C.c_int * 3),
                ("particle_radius", C.c_float), ("kernel_radius", C.c_float),
                ("kernel_factor", C.c_float), ("cell_size", C.c_float),
                ("rest_density", C.c_float), ("mass", C.c_float), ("gravity", C.c_float * 3),
                ("relaxation_epsilon", C.c_float), ("s_corr_dq", C.c_float),
                ("s_corr_k", C.c_float), ("s_corr_n", C.c_float), ("c_xsph", C.c_float),
                ("solid_contact", C.c_float), ("iterations", C.c_int),
                ("max_neighbors", C.c_int), ("clamp_cells", C.c_int), ("use_graph", C.c_int),
                ("grid_mode", C.c_int)]


GRID_AUTO, GRID_DENSE, GRID_HASHED = 0, 1, 2
LISTS_COLUMN, LISTS_COMPACT, LISTS_COMPACT_WIDE = 0, 1, 2


class PbfTuning(C.Structure):
    _fields_ = [("block", C.c_int), ("unroll", C.c_int), ("list_block", C.c_int), ("xsph_unroll", C.c_int),
                ("particles_per_thread", C.c_int), ("solver", C.c_int), ("solver_threads", C.c_int),
                ("list_format", C.c_int)]


class SandControls(C.Structure):
    _fields_ = [("player_position", C.c_float * 3), ("attract_flag", C.c_int), ("blow_flag", C.c_int),
                ("attract_radius", C.c_float), ("blow_radius", C.c_float), ("attract_coeff", C.c_float),
                ("blow_coeff", C.c_float), ("particle_diameter", C.c_float)]


# Every symbol include/lustrine_gb300.h declares, with its ctypes signature.
_P = C.c_void_p
_FP = C.POINTER(C.c_float)
_IP = C.POINTER(C.c_int)
_DP = C.POINTER(C.c_double)
SIGNATURES = {
    # layer 1: the reference's wrapper entry points
    "init_simulation": (None, [C.POINTER(SimulationParameters), C.POINTER(SimulationData),
                               C.POINTER(GridWrapper), C.c_int, C.POINTER(GridWrapper), C.c_int,
                               C.c_int]),
    "init_simulation_extra_parameters": (None, [C.POINTER(SimulationParameters),
                                                C.POINTER(SimulationData), C.POINTER(GridWrapper),
                                                C.c_int, C.POINTER(GridWrapper), C.c_int, C.c_int,
                                                C.c_float, C.c_int]),
    "simulate": (None, [C.c_float, C.c_bool, C.c_bool]),
    "simulate_no_flags": (None, [C.c_float]),
    "simulation_bind_positions_copy": (None, [_FP]),
    "cleanup_simulation": (None, []),
    "init_grid_box": (None, [C.POINTER(SimulationParameters), C.POINTER(GridWrapper), C.c_int,
                             C.c_int, C.c_int, Vec3, Color, C.c_int]),
    "get_num_sand_particles": (C.c_int, []),
    "get_grid_cell_size": (C.c_int, []),
    "set_simulate_function": (None, [C.c_int]),
    "lustrine_set_player_position": (None, [Vec3]),
    "query_cell_num_particles": (C.c_int, [Vec3, Vec3, C.c_bool]),
    "add_particle_source": (C.c_int, [C.POINTER(GridWrapper), Vec3, C.c_float, C.c_int]),
    "add_particle_sink": (C.c_int, [Vec3, Vec3, C.c_float]),
    "set_source_state": (None, [C.c_int, C.c_int]),
    "set_sink_state": (None, [C.c_int, C.c_int]),
    "get_source_spawned": (C.c_int, [C.c_int]),
    "get_sink_despawned": (C.c_int, [C.c_int]),
    "lustrine_last_status": (C.c_int, []),
    "lustrine_global_context": (_P, []),
    "lustrine_free_grid": (None, [C.POINTER(GridWrapper)]),
    "init_grid_magikavoxel": (None, [C.POINTER(GridWrapper), C.c_char_p, Vec3]),
    "create_grid": (None, [C.POINTER(GridWrapper), C.c_wchar_p, C.c_int, C.c_int]),
    "set_attract_blow_parameters": (None, [C.c_float, C.c_float, C.c_float, C.c_float]),
    "read_vox_scene": (None, [C.POINTER(BindingString), _P, C.c_int64]),
    "free_string": (None, [C.POINTER(BindingString)]),
    "test_allocate_1gb": (None, []),
    "test_deallocate_1gb": (None, []),
    # the Bullet world and the player: not built (each records LUSTRINE_ERR_UNSUPPORTED)
    "get_gravity": (Vec3, []),
    "set_gravity": (None, [Vec3]),
    "add_box": (C.c_int, [Vec3, C.c_bool, Vec3]),
    "add_capsule": (C.c_int, [Vec3, C.c_float, C.c_float]),
    "add_detector_block": (C.c_int, [Vec3, Vec3]),
    "check_collision": (C.c_int, [C.c_int, C.c_int]),
    "do_collide": (C.c_int, [C.c_int]),
    "do_collide_except_for": (C.c_int, [C.c_int, C.c_int]),
    "check_collisions": (None, [C.c_int, _IP, _IP]),
    "get_num_bodies": (C.c_int, []),
    "apply_impulse": (None, [C.c_int, Vec3, Vec3]),
    "get_position": (Vec3, [C.c_int]),
    "get_velocity": (Vec3, [C.c_int]),
    "set_velocity": (None, [C.c_int, Vec3]),
    "set_position": (None, [C.c_int, Vec3]),
    "add_velocity": (None, [C.c_int, Vec3]),
    "set_body_no_rotation": (None, [C.c_int]),
    "set_body_frixion": (None, [C.c_int, C.c_float]),
    "get_body_frixion": (C.c_float, [C.c_int]),
    "set_body_damping": (None, [C.c_int, C.c_float, C.c_float]),
    "get_body_damping": (C.c_float, [C.c_int]),
    "set_player_id": (None, [C.c_int]),
    "set_player_box_scale": (None, [Vec3]),
    "is_grounded": (C.c_int, [C.c_int]),
    "set_body_gravity": (None, [C.c_int, Vec3]),
    "set_body_no_collision_response": (None, [C.c_int]),
    "collide_with_player": (C.c_int, [C.c_int]),
    "enable_particles_bounding_boxes": (None, []),
    "disable_particles_bounding_boxes": (None, []),
    "set_player_particles_bounding_spheres_radius_placement": (None, [C.c_float]),
    # layer 2: context API
    "lustrine_pbf_params_reference": (None, [C.POINTER(PbfParams), C.c_int, C.c_int, C.c_int,
                                             C.c_float, C.c_float]),
    "lustrine_pbf_create": (C.c_int, [C.POINTER(PbfParams), C.c_int, C.c_int, C.POINTER(_P)]),
    "lustrine_pbf_destroy": (C.c_int, [_P]),
    "lustrine_batch_create": (C.c_int, [C.POINTER(PbfParams), C.c_int, _P, _P, _P, C.POINTER(_P)]),
    "lustrine_batch_set_solver": (C.c_int, [_P, C.c_int]),
    "lustrine_batch_get_solver": (C.c_int, [_P, _IP]),
    "lustrine_batch_onchip_layout": (C.c_int, [_P, _IP, _IP, _IP]),
    "lustrine_batch_set_onchip_threads": (C.c_int, [_P, C.c_int]),
    "lustrine_pbf_set_params": (C.c_int, [_P, C.POINTER(PbfParams)]),
    "lustrine_pbf_get_params": (C.c_int, [_P, C.POINTER(PbfParams)]),
    "lustrine_pbf_counts": (C.c_int, [_P, _IP, _IP]),
    "lustrine_pbf_upload": (C.c_int, [_P, _P, _P, _P]),
    "lustrine_pbf_upload_device": (C.c_int, [_P, _P, _P, _P]),
    "lustrine_pbf_upload_state_async": (C.c_int, [_P, _P, _P]),
    "lustrine_pbf_step": (C.c_int, [_P, C.c_float]),
    "lustrine_pbf_steps": (C.c_int, [_P, C.c_float, C.c_int]),
    "lustrine_pbf_synchronize": (C.c_int, [_P]),
    "lustrine_pbf_download": (C.c_int, [_P, _P, _P, _P, _P]),
    "lustrine_pbf_download_state_async": (C.c_int, [_P, _P, _P]),
    "lustrine_pbf_step_host": (C.c_int, [_P, C.c_float, _P, _P]),
    "lustrine_pbf_download_positions_f64": (C.c_int, [_P, _P]),
    "lustrine_pbf_neighbors": (C.c_int, [_P, _P, _P, C.c_int]),
    "lustrine_pbf_list_format": (C.c_int, [_P, _IP]),
    "lustrine_pbf_reduce": (C.c_int, [_P, _DP]),
    "lustrine_pbf_query_cell_count": (C.c_int, [_P, _FP, _FP, C.c_int, _IP]),
    "lustrine_pbf_reserve": (C.c_int, [_P, C.c_int]),
    "lustrine_pbf_spawn": (C.c_int, [_P, _P, _P, C.c_int]),
    "lustrine_pbf_despawn_cells": (C.c_int, [_P, _P, C.c_int, _IP]),
    "lustrine_pbf_set_count": (C.c_int, [_P, C.c_int]),
    "lustrine_pbf_status": (C.c_int, [_P]),
    "lustrine_pbf_stream": (C.c_int, [_P, C.POINTER(_P)]),
    "lustrine_pbf_launches_per_step": (C.c_int, [_P]),
    "lustrine_sand_controls_default": (None, [C.POINTER(SandControls), C.c_float]),
    "lustrine_pbf_set_sand_controls": (C.c_int, [_P, C.POINTER(SandControls)]),
    "lustrine_pbf_get_sand_controls": (C.c_int, [_P, C.POINTER(SandControls)]),
    "lustrine_pbf_get_attracted": (C.c_int, [_P, _P]),
    "lustrine_pbf_set_attracted": (C.c_int, [_P, _P]),
    "lustrine_pbf_profile_step": (C.c_int, [_P, C.c_float, _DP, _IP, C.c_int]),
    "lustrine_pbf_set_tuning": (C.c_int, [_P, C.POINTER(PbfTuning)]),
    "lustrine_pbf_get_tuning": (C.c_int, [_P, C.POINTER(PbfTuning)]),
    "lustrine_pbf_autotune": (C.c_int, [_P, C.c_float, C.c_int, C.POINTER(PbfTuning), _FP]),
    "lustrine_counting_sort": (C.c_int, [_P, _P, C.c_size_t, C.c_size_t, _P, _P]),
    "lustrine_counting_sort_noalloc": (C.c_int, [_P, _P, C.c_size_t, C.c_size_t, _P, _P]),
    "lustrine_error_string": (C.c_char_p, [C.c_int]),
}

_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load the CUDA library (building it with nvcc if it is missing or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing and not _build.up_to_date():
        _build.build()
    path = _build.LIB
    if not os.path.exists(path):
        raise RuntimeError(f"liblustrine_gb300.so not found at {path}; run lustrine_gb300.build")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(code: int, what: str = "") -> None:
    if code != LUSTRINE_OK:
        raise LustrineError(code, what)
