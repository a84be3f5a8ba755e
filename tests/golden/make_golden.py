"""Write the golden fixtures under tests/golden/ by running the reference's own
code, compiled from the reference tree by `make -C oracle ref`.

    python tests/golden/make_golden.py [--ref <reference tree>]   (default: $LUSTRINE_REFERENCE_DIR)

Fixtures (all from the reference binary, never from the restatement):
  counting_sort.npz   Sorting::counting_sort on the unit test's input
                      (experiments/unit_tests/main.cpp:46-89: 20,000 keys
                      rand() % 1987 from glibc's default seed).
  ref_c0_step.npz     one Lustrine::simulate step with simulate_fluid
                      (Simulate.cpp:27-115) of the 10,000-particle dam break
                      (20 x 25 x 20 block from (10, 0, 10), 40^3 box, r = 0.5,
                      h = 1.0, rho0 = 1, m = 1, g = -9.81, s_corr 0.1 / 4 /
                      0.2, jitter seed 0, dt = 1/60): input state, neighbour
                      lists (CSR, reference order), lambdas, x* and x, v.
  ref_solids_2step.npz  two steps of an 800-particle block (from (7, 3, 7),
                      resting on the solid tops) over a seeded
                      24 x 4 x 24 voxel heightmap (1,168 solids) in a
                      24 x 16 x 24 box, same parameters.
  ref_sand_steps.npz  the same scene stepped five times with simulate_sand
                      (Simulate.cpp:156-325, the wrapper's
                      set_simulate_function(0)): no flags; attract twice
                      with the player at (12, 6, 12); blow with the player
                      at (11, 5, 11.5); no flags.  Per step the state the
                      reference leaves (permuted into cell order), the
                      attracted flags and the neighbour lists (CSR, the
                      reference's push order, itself included twice), as
                      x1..x5, v1..v5, att1..att5, nbr_off1.., nbr1..
  wrapper_symbols.txt  the names of every extern "C" entry point the
                      reference's wrapper header declares
                      (src/LustrineWrapper.hpp), one per line.
  vox/*.vox, vox_ref.npz  small MagicaVoxel files written here from the
                      published chunk format (SIZE, XYZI, RGBA, PACK; an empty
                      first model; a voxel listed twice; colour index 255),
                      and what the reference's loader init_grid_from_magika_voxel
                      (VoxelLoader.cpp:48-99) makes of each: cells, colours,
                      occupied count; with the palettes written.
"""
from __future__ import annotations

import argparse
import ctypes
import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from lustrine_gb300 import scenes  # noqa: E402

PHYS = dict(rest_density=1.0, mass=1.0, gravity=(0.0, -9.81, 0.0), eps=10.0, dq=0.2, k=0.1, n=4.0)


def csr(cnt, idx):
    off = np.zeros(len(cnt) + 1, np.int64)
    off[1:] = np.cumsum(cnt)
    flat = np.concatenate([idx[i, : cnt[i]] for i in range(len(cnt))]) if len(cnt) else np.zeros(0)
    return off.astype(np.int32), flat.astype(np.int32)


def glibc_rand_keys(num, mod):
    libc = ctypes.CDLL("libc.so.6")
    libc.srand(1)
    return np.array([libc.rand() % mod for _ in range(num)], np.int32)


def make_counting_sort(R):
    keys = glibc_rand_keys(20000, 1987)
    perm = R.counting_sort(keys, 1987)
    np.savez_compressed(os.path.join(HERE, "counting_sort.npz"), keys=keys, num_cells=1987,
                        perm=perm)


def set_phys(R):
    R.set_params(PHYS["rest_density"], PHYS["mass"], PHYS["gravity"], PHYS["eps"], PHYS["dq"],
                 PHYS["k"], PHYS["n"])


def make_c0(R):
    sc = scenes.config0(seed=0)
    n = R.init(40, 40, 40, (20, 25, 20), (10, 0, 10))
    assert n == sc.n
    x0_ref, _, _, _ = R.state()
    assert np.array_equal(x0_ref, scenes.lattice((20, 25, 20), (10, 0, 10)))
    set_phys(R)
    v0 = np.zeros_like(sc.x)
    R.set_state(sc.x, v0)
    dt = np.float32(1.0 / 60.0)
    R.step(dt)
    x, xs, v, lam = R.state()
    cnt, idx = R.neighbors(cap=256)
    off, flat = csr(cnt, idx)
    np.savez_compressed(os.path.join(HERE, "ref_c0_step.npz"), domain=np.array([40, 40, 40]),
                        x0=sc.x, v0=v0, dt=dt, x=x, xs=xs, v=v, lam=lam, nbr_off=off, nbr=flat,
                        grid=np.array([R.info(7), R.info(8), R.info(9)]), floats=R.floats(),
                        ptrs=np.array([R.info(k) for k in range(5)]))


def solid_grid(seed=7):
    rng = np.random.default_rng(seed)
    GX, GY, GZ = 24, 4, 24
    H = rng.integers(1, 4, size=(GX, GZ))
    cells = np.zeros((GX, GY, GZ), np.int32)
    for xx in range(GX):
        for zz in range(GZ):
            cells[xx, : H[xx, zz], zz] = 1
    return cells, rng


def make_solids(R):
    cells, rng = solid_grid()
    n = R.init(24, 16, 24, (10, 8, 10), (7, 3, 7), solids=[(cells.shape, (0, 0, 0), cells)])
    set_phys(R)
    x0_ref, _, _, _ = R.state()
    x0 = (x0_ref + rng.uniform(-0.05, 0.05, x0_ref.shape)).astype(np.float32)
    v0 = np.zeros_like(x0)
    R.set_state(x0, v0)
    solid = R.solids()
    dt = np.float32(1.0 / 60.0)
    out = dict(domain=np.array([24, 16, 24]), x0=x0, v0=v0, solid=solid, dt=dt, cells=cells,
               ptrs=np.array([R.info(k) for k in range(5)]))
    for s in (1, 2):
        R.step(dt)
        x, xs, v, lam = R.state()
        cnt, idx = R.neighbors(cap=256)
        off, flat = csr(cnt, idx)
        out.update({f"x{s}": x, f"v{s}": v, f"lam{s}": lam, f"nbr_off{s}": off, f"nbr{s}": flat})
    np.savez_compressed(os.path.join(HERE, "ref_solids_2step.npz"), **out)
    return n


SAND_PLAN = (dict(), dict(attract=True, player=(12.0, 6.0, 12.0)), dict(attract=True, player=(12.0, 6.0, 12.0)),
             dict(blow=True, player=(11.0, 5.0, 11.5)), dict())


def make_sand(R):
    """Five simulate_sand calls on the solids scene.  simulate_sand keeps the
    previous call's attract flag in a function static, false at process start:
    run this once per process."""
    cells, rng = solid_grid()
    n = R.init(24, 16, 24, (10, 8, 10), (7, 3, 7), solids=[(cells.shape, (0, 0, 0), cells)])
    set_phys(R)
    x0_ref, _, _, _ = R.state()
    x0 = (x0_ref + rng.uniform(-0.05, 0.05, x0_ref.shape)).astype(np.float32)
    v0 = np.zeros_like(x0)
    R.set_state(x0, v0)
    R.set_step_function(1)
    dt = np.float32(1.0 / 60.0)
    out = dict(domain=np.array([24, 16, 24]), x0=x0, v0=v0, solid=R.solids(), dt=dt,
               diameter=np.float32(R.diameter()),
               player=np.array([c.get("player", (0.0, 0.0, 0.0)) for c in SAND_PLAN], np.float32),
               attract=np.array([c.get("attract", False) for c in SAND_PLAN], np.int32),
               blow=np.array([c.get("blow", False) for c in SAND_PLAN], np.int32))
    for s, c in enumerate(SAND_PLAN, start=1):
        R.set_sand_controls(O.sand_controls(diameter=R.diameter(), **c))
        R.step(dt)
        x, _, v, _ = R.state()
        cnt, idx = R.neighbors(cap=96)
        off, flat = csr(cnt, idx)
        out.update({f"x{s}": x, f"v{s}": v, f"att{s}": R.attracted(), f"nbr_off{s}": off, f"nbr{s}": flat})
    np.savez_compressed(os.path.join(HERE, "ref_sand_steps.npz"), **out)
    return n


def _vox_chunk(cid, content=b"", children=b""):
    return cid + struct.pack("<II", len(content), len(children)) + content + children


def write_vox(path, models, rgba, version=150, extra=b""):
    """A MagicaVoxel file: models = [((X, Y, Z), [(x, y, z, colour), ...]), ...]."""
    kids = extra
    for size, vox in models:
        kids += _vox_chunk(b"SIZE", struct.pack("<III", *size))
        kids += _vox_chunk(b"XYZI", struct.pack("<I", len(vox)) + b"".join(bytes(v) for v in vox))
    kids += _vox_chunk(b"RGBA", np.ascontiguousarray(rgba, np.uint8).tobytes())
    with open(path, "wb") as f:
        f.write(b"VOX " + struct.pack("<I", version) + _vox_chunk(b"MAIN", b"", kids))


def make_vox(R):
    rng = np.random.default_rng(11)
    d = os.path.join(HERE, "vox")
    os.makedirs(d, exist_ok=True)
    files = {}
    # a 5 x 4 x 6 model, ~40 % occupied, colours 1..255
    pal = rng.integers(0, 256, size=(256, 4), dtype=np.uint8)
    vox = [(x, y, z, int(rng.integers(1, 256))) for x in range(5) for y in range(4) for z in range(6)
           if rng.random() < 0.4]
    files["box.vox"] = (pal, [((5, 4, 6), vox)], 150, b"")
    # an empty first model (skipped), a PACK chunk, version 200
    pal2 = rng.integers(0, 256, size=(256, 4), dtype=np.uint8)
    vox2 = [(x, y, z, 1 + (x + 2 * y + 3 * z) % 7) for x in range(4) for y in range(2) for z in range(3)
            if (x + y + z) % 2 == 0]
    files["empty_first.vox"] = (pal2, [((3, 3, 3), []), ((4, 2, 3), vox2)], 200,
                                _vox_chunk(b"PACK", struct.pack("<I", 2)))
    # a voxel listed twice (the later colour stays), colour index 255, a second model ignored
    vox3 = [(0, 0, 0, 3), (1, 2, 1, 255), (0, 0, 0, 9), (2, 0, 1, 1)]
    files["dup.vox"] = (pal, [((3, 3, 2), vox3), ((2, 2, 2), [(1, 1, 1, 5)])], 150, b"")
    out = {}
    for name, (p, models, version, extra) in files.items():
        path = os.path.join(d, name)
        write_vox(path, models, p, version, extra)
        cells, colors, occ = R.load_vox(path)
        key = name[:-4]
        out.update({f"{key}_cells": cells, f"{key}_colors": colors, f"{key}_occupied": occ, f"{key}_rgba": p})
    np.savez_compressed(os.path.join(HERE, "vox_ref.npz"), **out)


def make_wrapper_symbols(ref_root):
    """The reference wrapper's extern "C" names, read from its header (lines
    commented out with // are skipped)."""
    import re
    names = []
    for line in open(os.path.join(ref_root, "src", "LustrineWrapper.hpp")):
        code = line.split("//", 1)[0]
        m = re.search(r'extern\s+"C"\s+\w+\s+[\w:<>\s\*]+?\b(\w+)\s*\(', code)
        if m:
            names.append(m.group(1))
    with open(os.path.join(HERE, "wrapper_symbols.txt"), "w") as f:
        f.write("\n".join(names) + "\n")
    return names


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("LUSTRINE_REFERENCE_DIR"))
    ap.add_argument("--symbols-only", action="store_true",
                    help="write wrapper_symbols.txt only (no reference build)")
    a = ap.parse_args()
    if not a.ref or not os.path.isdir(os.path.join(a.ref, "src")):
        raise SystemExit("the reference tree is not available (--ref or LUSTRINE_REFERENCE_DIR); fixtures are committed")
    make_wrapper_symbols(a.ref)
    if a.symbols_only:
        return
    path = O.build_ref(a.ref)
    if not path:
        raise SystemExit("the reference tree is not available; fixtures are committed")
    R = O.Reference(path)
    make_counting_sort(R)
    make_c0(R)
    make_solids(R)
    make_sand(R)
    make_vox(R)
    R.L.ref_free()
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
