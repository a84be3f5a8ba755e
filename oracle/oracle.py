"""ctypes bindings for the CPU oracle (oracle/_build/liborc.so) and, where it
was built, the reference's own fluid path (oracle/_ref/libref.so).

TEST INFRASTRUCTURE.  Only tests/, ``__graft_entry__.smoke()`` and the CPU
baseline leg of bench.py import this module; the product package
(lustrine_gb300) never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORC_SO = os.path.join(HERE, "_build", "liborc.so")
REF_SO = os.path.join(HERE, "_ref", "libref.so")


class OrcParams(C.Structure):
    """Mirror of ``orc_params`` in pbf_oracle.h."""

    _fields_ = [
        ("domain", C.c_float * 3),
        ("grid", C.c_int * 3),
        ("cell_size", C.c_float),
        ("particle_radius", C.c_float),
        ("kernel_radius", C.c_float),
        ("kernel_factor", C.c_float),
        ("cubic_k", C.c_float),
        ("cubic_l", C.c_float),
        ("rest_density", C.c_float),
        ("mass", C.c_float),
        ("gravity", C.c_float * 3),
        ("relaxation_epsilon", C.c_float),
        ("s_corr_dq", C.c_float),
        ("s_corr_k", C.c_float),
        ("s_corr_n", C.c_float),
        ("c_xsph", C.c_float),
        ("solid_contact", C.c_float),
        ("iterations", C.c_int),
        ("clamp_cells", C.c_int),
        ("jacobi", C.c_int),
    ]


class OrcSandControls(C.Structure):
    """Mirror of ``orc_sand_controls`` in pbf_oracle.h."""

    _fields_ = [
        ("player_position", C.c_float * 3),
        ("attract_flag", C.c_int),
        ("blow_flag", C.c_int),
        ("prev_attract_flag", C.c_int),
        ("attract_radius", C.c_float),
        ("blow_radius", C.c_float),
        ("attract_coeff", C.c_float),
        ("blow_coeff", C.c_float),
        ("particle_diameter", C.c_float),
    ]


def sand_controls(player=(0.0, 0.0, 0.0), attract=False, blow=False, prev_attract=False,
                  attract_radius=1.5, blow_radius=2.0, attract_coeff=1000.0, blow_coeff=500.0,
                  diameter=1.0) -> OrcSandControls:
    """simulate_sand's controls; the radii and coefficients default to the
    reference's (Simulation.hpp:239-242)."""
    c = OrcSandControls()
    c.player_position[:] = [float(a) for a in player]
    c.attract_flag, c.blow_flag, c.prev_attract_flag = int(attract), int(blow), int(prev_attract)
    c.attract_radius, c.blow_radius = attract_radius, blow_radius
    c.attract_coeff, c.blow_coeff = attract_coeff, blow_coeff
    c.particle_diameter = diameter
    return c


def build(force: bool = False) -> str:
    """Compile the C restatement with the committed Makefile."""
    if force or not os.path.exists(ORC_SO) or os.path.getmtime(ORC_SO) < max(
        os.path.getmtime(os.path.join(HERE, f))
        for f in ("pbf_oracle.c", "pbf_oracle.h", "pbf_mode_p.inc", "sand_oracle.inc")
    ):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return ORC_SO


def reference_dir() -> str | None:
    """The reference tree named by LUSTRINE_REFERENCE_DIR, or None when the
    variable is unset or names no tree with a src/ folder."""
    d = os.environ.get("LUSTRINE_REFERENCE_DIR")
    return d if d and os.path.isdir(os.path.join(d, "src")) else None


def build_ref(ref_root: str | None = None) -> str | None:
    """Compile the reference's fluid path from the reference tree (ref_root,
    else LUSTRINE_REFERENCE_DIR).  Returns the library path, or the one built
    earlier, or None."""
    ref_root = ref_root or reference_dir()
    if not ref_root or not os.path.isdir(os.path.join(ref_root, "src")):
        return REF_SO if os.path.exists(REF_SO) else None
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref_root}"], check=True)
    return REF_SO


_F = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_D = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_I = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def _opt(ptr_type):
    """An ndpointer that also accepts None."""

    class _Opt(ptr_type):
        @classmethod
        def from_param(cls, obj):
            if obj is None:
                return None
            return super().from_param(obj)

    return _Opt


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(ORC_SO)
        P = C.POINTER(OrcParams)
        L.orc_params_reference.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float]
        L.orc_counting_sort.argtypes = [_I, _I, C.c_size_t, C.c_size_t, _I]
        L.orc_compat_step.argtypes = [P, C.c_float, C.c_int, C.c_int, _F, _F, _F, _opt(_F),
                                      _F, _opt(_I), _opt(_I), C.c_int]
        L.orc_compat_neighbors.argtypes = [P, C.c_int, C.c_int, _F, _opt(_F), _opt(_I),
                                           _opt(_I), C.c_int]
        L.orc_pbf_step_d.argtypes = [P, C.c_double, C.c_int, C.c_int, _D, _D, _opt(_D),
                                     _opt(_D), _opt(_D), _opt(_I)]
        L.orc_pbf_step_f.argtypes = [P, C.c_float, C.c_int, C.c_int, _F, _F, _opt(_F),
                                     _opt(_F), _opt(_F), _opt(_I)]
        L.orc_pbf_density_d.argtypes = [P, C.c_int, C.c_int, _D, _opt(_D), _D]
        L.orc_pbf_lambda_d.argtypes = [P, C.c_int, C.c_int, _D, _opt(_D), _opt(_D), _opt(_D)]
        L.orc_sand_step.argtypes = [P, C.POINTER(OrcSandControls), C.c_float, C.c_int, C.c_int, _F, _F,
                                    _I, _opt(_F), _opt(_I), _opt(_I), C.c_int, _opt(_F)]
        _lib = L
    return _lib


def reference_params(X, Y, Z, radius=0.5, scale=2.0) -> OrcParams:
    p = OrcParams()
    lib().orc_params_reference(C.byref(p), X, Y, Z, radius, scale)
    return p


def counting_sort(keys: np.ndarray, num_cells: int) -> np.ndarray:
    keys = np.ascontiguousarray(keys, dtype=np.int32)
    counts = np.zeros(num_cells + 1, np.int32)
    out = np.zeros(len(keys), np.int32)
    lib().orc_counting_sort(counts, keys, len(keys), num_cells, out)
    return out


def _solid_arg(solid, dtype):
    if solid is None or len(solid) == 0:
        return None, 0
    s = np.ascontiguousarray(solid, dtype=dtype).reshape(-1)
    return s, len(s) // 3


def compat_step(p: OrcParams, dt, x, v, solid=None, lambdas=None, cap=256):
    """One reference-semantics step (mode R).  Returns dict with x, xs, v,
    lambdas (n + ns), nbr_count, nbr_idx (n x cap)."""
    x = np.array(x, np.float32).reshape(-1)
    v = np.array(v, np.float32).reshape(-1)
    n = len(x) // 3
    s, ns = _solid_arg(solid, np.float32)
    xs = x.copy()
    lam = np.zeros(n + ns + 1, np.float32) if lambdas is None else np.array(lambdas, np.float32)
    cnt = np.zeros(n, np.int32)
    idx = np.full(n * cap, -1, np.int32)
    rc = lib().orc_compat_step(C.byref(p), dt, n, ns, x, xs, v, s, lam, cnt, idx, cap)
    if rc:
        raise RuntimeError(f"orc_compat_step failed: {rc}")
    return dict(x=x.reshape(n, 3), xs=xs.reshape(n, 3), v=v.reshape(n, 3), lambdas=lam,
                nbr_count=cnt, nbr_idx=idx.reshape(n, cap))


def compat_neighbors(p: OrcParams, xs, solid=None, cap=256):
    xs = np.ascontiguousarray(xs, np.float32).reshape(-1)
    n = len(xs) // 3
    s, ns = _solid_arg(solid, np.float32)
    cnt = np.zeros(n, np.int32)
    idx = np.full(n * cap, -1, np.int32)
    rc = lib().orc_compat_neighbors(C.byref(p), n, ns, xs, s, cnt, idx, cap)
    if rc:
        raise RuntimeError(f"orc_compat_neighbors failed: {rc}")
    return cnt, idx.reshape(n, cap)


def pbf_step(p: OrcParams, dt, x, v, solid=None, dtype=np.float64):
    """One mode-P step in float64 (default) or float32.  Returns dict."""
    x = np.array(x, dtype).reshape(-1)
    v = np.array(v, dtype).reshape(-1)
    n = len(x) // 3
    s, ns = _solid_arg(solid, dtype)
    lam = np.zeros(n, dtype)
    rho = np.zeros(n, dtype)
    cnt = np.zeros(n, np.int32)
    fn = lib().orc_pbf_step_d if dtype == np.float64 else lib().orc_pbf_step_f
    rc = fn(C.byref(p), dt, n, ns, x, v, s, lam, rho, cnt)
    if rc:
        raise RuntimeError(f"orc_pbf_step failed: {rc}")
    return dict(x=x.reshape(n, 3), v=v.reshape(n, 3), lambdas=lam, density=rho, nbr_count=cnt)


def pbf_density(p: OrcParams, xs, solid=None):
    xs = np.ascontiguousarray(xs, np.float64).reshape(-1)
    n = len(xs) // 3
    s, ns = _solid_arg(solid, np.float64)
    rho = np.zeros(n, np.float64)
    rc = lib().orc_pbf_density_d(C.byref(p), n, ns, xs, s, rho)
    if rc:
        raise RuntimeError(f"orc_pbf_density_d failed: {rc}")
    return rho


def pbf_lambda(p: OrcParams, xs, solid=None):
    xs = np.ascontiguousarray(xs, np.float64).reshape(-1)
    n = len(xs) // 3
    s, ns = _solid_arg(solid, np.float64)
    rho = np.zeros(n, np.float64)
    lam = np.zeros(n, np.float64)
    rc = lib().orc_pbf_lambda_d(C.byref(p), n, ns, xs, s, lam, rho)
    if rc:
        raise RuntimeError(f"orc_pbf_lambda_d failed: {rc}")
    return lam, rho


def sand_step(p: OrcParams, ctl: OrcSandControls, dt, x, v, attracted=None, solid=None, cap=64):
    """One call of the reference's sand step.  The state comes back permuted
    into cell order, as the reference leaves it.  Returns dict with x, v,
    attracted, nbr_count, nbr_idx (n x cap; itself twice, static k as n + k)
    and xs (the predicted positions the step binned, sorted order)."""
    x = np.array(x, np.float32).reshape(-1)
    v = np.array(v, np.float32).reshape(-1)
    n = len(x) // 3
    att = np.zeros(n, np.int32) if attracted is None else np.array(attracted, np.int32)
    s, ns = _solid_arg(solid, np.float32)
    cnt = np.zeros(n, np.int32)
    idx = np.full(n * cap, -1, np.int32)
    xs = np.zeros(3 * max(n, 1), np.float32)
    rc = lib().orc_sand_step(C.byref(p), C.byref(ctl), dt, n, ns, x, v, att, s, cnt, idx, cap, xs)
    if rc:
        raise RuntimeError(f"orc_sand_step failed: {rc}")
    return dict(x=x.reshape(n, 3), v=v.reshape(n, 3), attracted=att, nbr_count=cnt,
                nbr_idx=idx.reshape(n, cap), xs=xs[: 3 * n].reshape(n, 3))


# ---------------------------------------------------------------- reference --

class Reference:
    """The reference's own fluid step, compiled from its sources (oracle/_ref)."""

    def __init__(self, path: str = REF_SO):
        L = C.CDLL(path)
        L.ref_init.argtypes = [C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_int, C.c_int,
                               C.c_int, _F, C.c_int, _opt(_I), _opt(_F), _opt(_I)]
        L.ref_init.restype = C.c_int
        L.ref_set_params.argtypes = [C.c_float, C.c_float, _F, C.c_float, C.c_float, C.c_float,
                                     C.c_float]
        L.ref_info.argtypes = [C.c_int]
        L.ref_info.restype = C.c_longlong
        L.ref_get_floats.argtypes = [_F]
        L.ref_set_state.argtypes = [_F, _F]
        L.ref_get_state.argtypes = [_opt(_F), _opt(_F), _opt(_F), _opt(_F)]
        L.ref_get_solids.argtypes = [_F]
        L.ref_step.argtypes = [C.c_float]
        L.ref_neighbors.argtypes = [_I, _I, C.c_int]
        L.ref_neighbors.restype = C.c_int
        L.ref_counting_sort.argtypes = [_I, _I, C.c_size_t, C.c_size_t, _I]
        L.ref_set_step_function.argtypes = [C.c_int]
        L.ref_set_sand_controls.argtypes = [_F, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float,
                                            C.c_float]
        L.ref_get_attracted.argtypes = [_I]
        L.ref_set_attracted.argtypes = [_I]
        L.ref_get_float.argtypes = [C.c_int]
        L.ref_get_float.restype = C.c_float
        L.ref_load_vox.argtypes = [C.c_char_p, _I, _I, _F, C.c_int]
        L.ref_load_vox.restype = C.c_int
        self.L = L

    def init(self, X, Y, Z, block, block_pos, radius=0.5, scale=2.0, solids=()):
        """solids: sequence of (dims(3), pos(3), cells (dims product ints))."""
        dims = np.array([d for s in solids for d in s[0]], np.int32) if solids else None
        pos = np.array([c for s in solids for c in s[1]], np.float32) if solids else None
        cells = (np.concatenate([np.asarray(s[2], np.int32).reshape(-1) for s in solids])
                 if solids else None)
        n = self.L.ref_init(X, Y, Z, radius, scale, block[0], block[1], block[2],
                            np.array(block_pos, np.float32), len(solids), dims, pos, cells)
        self.n = n
        self.ns = int(self.L.ref_info(6))
        return n

    def set_params(self, rest_density, mass, gravity, eps, dq, k, n):
        self.L.ref_set_params(rest_density, mass, np.array(gravity, np.float32), eps, dq, k, n)

    def info(self, which):
        return int(self.L.ref_info(which))

    def floats(self):
        f = np.zeros(6, np.float32)
        self.L.ref_get_floats(f)
        return f

    def set_state(self, x, v):
        self.L.ref_set_state(np.ascontiguousarray(x, np.float32).reshape(-1),
                             np.ascontiguousarray(v, np.float32).reshape(-1))

    def state(self):
        n = self.n
        x, xs, v = (np.zeros(3 * n, np.float32) for _ in range(3))
        lam = np.zeros(n, np.float32)
        self.L.ref_get_state(x, xs, v, lam)
        return x.reshape(n, 3), xs.reshape(n, 3), v.reshape(n, 3), lam

    def solids(self):
        s = np.zeros(3 * max(self.ns, 1), np.float32)
        self.L.ref_get_solids(s)
        return s[: 3 * self.ns].reshape(self.ns, 3)

    def step(self, dt):
        self.L.ref_step(dt)

    def neighbors(self, cap=256):
        cnt = np.zeros(self.n, np.int32)
        idx = np.full(self.n * cap, -1, np.int32)
        rc = self.L.ref_neighbors(cnt, idx, cap)
        if rc:
            raise RuntimeError("reference neighbour list exceeds cap")
        return cnt, idx.reshape(self.n, cap)

    def counting_sort(self, keys, num_cells):
        keys = np.ascontiguousarray(keys, np.int32)
        counts = np.zeros(num_cells + 1, np.int32)
        out = np.zeros(len(keys), np.int32)
        self.L.ref_counting_sort(counts, keys, len(keys), num_cells, out)
        return out

    def set_step_function(self, which):
        """0: simulate_fluid, 1: simulate_sand."""
        self.L.ref_set_step_function(which)

    def set_sand_controls(self, ctl: OrcSandControls):
        self.L.ref_set_sand_controls(np.array(ctl.player_position[:], np.float32), ctl.attract_flag,
                                     ctl.blow_flag, ctl.attract_radius, ctl.blow_radius,
                                     ctl.attract_coeff, ctl.blow_coeff)

    def attracted(self):
        a = np.zeros(self.n, np.int32)
        self.L.ref_get_attracted(a)
        return a

    def set_attracted(self, a):
        self.L.ref_set_attracted(np.ascontiguousarray(a, np.int32))

    def diameter(self):
        return float(self.L.ref_get_float(0))

    def load_vox(self, path, cap=1 << 24):
        """init_grid_from_magika_voxel: (cells[X, Y, Z], colors[X, Y, Z, 4], occupied)."""
        dims = np.zeros(3, np.int32)
        cells = np.zeros(cap, np.int32)
        colors = np.zeros(4 * cap, np.float32)
        occ = self.L.ref_load_vox(os.fsencode(str(path)), dims, cells, colors, cap)
        if occ < 0:
            raise RuntimeError("voxel grid larger than cap")
        X, Y, Z = (int(a) for a in dims)
        n = X * Y * Z
        return cells[:n].reshape(X, Y, Z), colors[:4 * n].reshape(X, Y, Z, 4), occ
