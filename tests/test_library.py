"""The C-ABI library without a GPU: it builds for sm_103a, loads, exports
every symbol include/lustrine_gb300.h declares, and its structs have the
reference's layouts.  No compute call is made here."""
import ctypes as C
import os
import re
import subprocess

import numpy as np

from conftest import ROOT


def _declared_symbols():
    text = open(os.path.join(ROOT, "include", "lustrine_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"LUSTRINE_API\s+[\w\s\*]+?\b(\w+)\s*\(", text)))


def test_library_builds_and_exports_every_declared_symbol():
    from lustrine_gb300 import _lib
    lib = _lib.load()
    declared = _declared_symbols()
    assert len(declared) >= 30
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing
    # the Python binding covers the same set
    assert set(declared) <= set(_lib.SIGNATURES), set(declared) - set(_lib.SIGNATURES)


def _exported_symbols():
    from lustrine_gb300 import _lib
    _lib.load()
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.library_path()], capture_output=True,
                         text=True, check=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if ln.strip()}


def test_library_exports_every_reference_wrapper_symbol():
    """nm -D of the library is a superset of the extern "C" names the
    reference's wrapper header declares (tests/golden/wrapper_symbols.txt,
    written from src/LustrineWrapper.hpp by make_golden.py), so a binding
    built for the reference's library finds every entry point here."""
    ref = [ln.strip() for ln in open(os.path.join(ROOT, "tests", "golden", "wrapper_symbols.txt")) if ln.strip()]
    assert len(ref) == 54
    missing = sorted(set(ref) - _exported_symbols())
    assert not missing, missing
    assert set(ref) <= set(_declared_symbols())


def test_unbuilt_wrapper_entry_points_record_unsupported():
    """The Bullet/player entry points and read_vox_scene answer with zeros and
    record LUSTRINE_ERR_UNSUPPORTED (no GPU involved); set_attract_blow_parameters
    before init records LUSTRINE_ERR_NO_SIMULATION."""
    from lustrine_gb300 import _lib
    lib = _lib.load()
    v = lib.get_gravity()
    assert (v.x, v.y, v.z) == (0.0, 0.0, 0.0) and lib.lustrine_last_status() == 6
    assert lib.add_box(_lib.Vec3(1, 2, 3), True, _lib.Vec3(1, 1, 1)) == 0 and lib.lustrine_last_status() == 6
    assert lib.get_body_frixion(0) == 0.0 and lib.lustrine_last_status() == 6
    idx = np.full(4, 7, np.int32)
    size = np.full(1, 5, np.int32)
    lib.check_collisions(0, idx.ctypes.data_as(C.POINTER(C.c_int)), size.ctypes.data_as(C.POINTER(C.c_int)))
    assert size[0] == 0 and lib.lustrine_last_status() == 6
    s = _lib.BindingString(3, b"abc")
    lib.read_vox_scene(C.byref(s), None, 0)
    assert s.length == 0 and not s.data and lib.lustrine_last_status() == 6
    lib.free_string(C.byref(s))
    assert lib.lustrine_last_status() == 0
    lib.cleanup_simulation()
    lib.set_attract_blow_parameters(1.0, 2.0, 3.0, 4.0)
    assert lib.lustrine_last_status() == 7


def test_struct_layouts_match_reference_abi():
    from lustrine_gb300._lib import (Color, GridWrapper, PbfParams, SimulationData,
                                     SimulationParameters, Vec3)
    assert C.sizeof(SimulationParameters) == 20   # 3 ints + 2 floats (Simulation.hpp:83-92)
    assert C.sizeof(SimulationData) == 24         # 6 ints (LustrineWrapper.hpp:30-41)
    assert C.sizeof(Color) == 16 and C.sizeof(Vec3) == 12
    # GridWrapper (LustrineWrapper.hpp:62-74) on LP64: 2 pointers, Color, Vec3, bool, 6 ints
    assert GridWrapper.color.offset == 16 and GridWrapper.position.offset == 32
    assert GridWrapper.has_one_color_per_cell.offset == 44 and GridWrapper.X.offset == 48
    assert GridWrapper.type.offset == 68 and C.sizeof(GridWrapper) == 72
    assert C.sizeof(PbfParams) == 4 * 25  # 25 four-byte fields


def test_error_strings_and_reference_params_need_no_gpu():
    from lustrine_gb300 import _lib, reference_params
    lib = _lib.load()
    assert lib.lustrine_error_string(4) == b"neighbour list capacity exceeded"
    p = reference_params(40, 40, 40)
    # Lustrine.cpp:545-546 with kernel_radius_scale 2 and Simulation.hpp defaults
    assert p.kernel_radius == 1.0 and p.cell_size == 1.0 and p.kernel_factor == 0.5
    assert p.rest_density == 24.0 and p.mass == 5.0 and p.gravity[1] == -10.0


def test_scenes_match_config_shapes():
    from lustrine_gb300 import scenes
    c0 = scenes.config0()
    assert c0.n == 10_000 and c0.domain == (40, 40, 40)
    assert np.abs(c0.x - scenes.lattice((20, 25, 20), (10, 0, 10))).max() <= 0.05 + 1e-6
    c1 = scenes.config1()
    assert c1.n == 262_144 and 47_500 <= c1.ns <= 52_500
    assert (c1.solid.min(0) >= 0).all() and (c1.solid.max(0) <= np.array(c1.domain)).all()
    counts = scenes.batched_counts()
    assert len(counts) == 512 and counts.min() >= 1024 and counts.max() <= 65536
    s = scenes.batched_scene(1500, np.random.default_rng(0))
    assert s.n == 1500 and (s.x.max(0) < np.array(s.domain)).all()


def test_bench_workloads_have_their_quoted_sizes():
    """The seeded workloads the bench measures: config 3's 512 scenes hold
    7,546,040 particles, 1,029 to 65,482 a scene (every scene below 65,536,
    so the batch takes 16-bit compact entries), each inside its box; config
    2 holds 2,097,152 and config 4 4,194,304 particles inside their domains."""
    from lustrine_gb300 import scenes
    c3 = scenes.config3()
    counts = np.array([s.n for s in c3])
    assert len(c3) == 512 and counts.sum() == 7_546_040
    assert counts.min() == 1_029 and counts.max() == 65_482 < 65_536
    for s in c3[:64]:
        assert (s.x.min(0) > 0).all() and (s.x.max(0) < np.array(s.domain)).all()
    c2 = scenes.config2()
    assert c2.n == 2_097_152 and (c2.x.max(0) < np.array(c2.domain)).all()
    c4 = scenes.config4()
    assert c4.n == 4_194_304 and (c4.x.min(0) > 0).all() and (c4.x.max(0) < np.array(c4.domain)).all()


def test_rest_lattice_mass_puts_the_rest_lattice_at_rest_density():
    """The PBF scenes' default mass: the poly6 density of the rest lattice
    equals the rest density, for h at the spacing and beyond it."""
    from lustrine_gb300 import pbf_params, rest_lattice_mass
    for rho0, h, spacing in ((1.0, 1.0, 1.0), (1.0, 2.0, 1.0), (24.0, 1.5, 0.5)):
        m = rest_lattice_mass(rho0, h, spacing)
        k = np.arange(-6, 7)
        r2 = (k[:, None, None] ** 2 + k[None, :, None] ** 2 + k[None, None, :] ** 2) * spacing ** 2
        hd = np.clip(h * h - r2, 0.0, None)
        rho = m * 315.0 / (64.0 * np.pi * h ** 9) * (hd ** 3).sum()
        assert abs(rho - rho0) <= 1e-12 * rho0
    assert abs(rest_lattice_mass(1.0, 1.0, 1.0) - 64.0 * np.pi / 315.0) < 1e-15
    assert abs(pbf_params(40, 40, 40).mass - np.float32(64.0 * np.pi / 315.0)) == 0
    assert pbf_params(40, 40, 40, mass=1.0).mass == 1.0


def _header_struct_fields(name):
    text = open(os.path.join(ROOT, "include", "lustrine_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    body = re.search(r"typedef struct " + name + r"\s*\{(.*?)\}\s*" + name + ";", text, re.S).group(1)
    return [re.findall(r"(\w+)\s*(?:\[\d+\])?\s*;", d)[0] for d in body.split(";") if d.strip()
            for d in [d + ";"]]


def test_ctypes_structs_follow_the_header():
    """The Python host side's ctypes structs list the header's fields in the
    header's order (the launch shape, the sand controls)."""
    from lustrine_gb300._lib import PbfTuning, SandControls
    for cls, name in ((PbfTuning, "lustrine_pbf_tuning"), (SandControls, "lustrine_sand_controls")):
        assert [f[0] for f in cls._fields_] == _header_struct_fields(name), name
    assert C.sizeof(PbfTuning) == 32
