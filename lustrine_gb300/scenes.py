"""Seeded synthetic scenes for the five benchmark configurations.

No dataset is involved: every scene is a jittered particle lattice (a dam
break) and, for the voxel-solid scene, a seeded value-noise heightmap
voxelised at unit cells.  Lattices follow the reference's particle order
(init_chunk_from_grid, Lustrine.cpp:694-716: x outer, y, z inner; position =
index * diameter + grid position + diameter / 2).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Scene:
    name: str
    domain: tuple                    # box X, Y, Z (ints)
    x: np.ndarray                    # (n, 3) float32 fluid positions
    solid: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.float32))
    dt: float = 1.0 / 60.0
    iterations: int = 4
    steps: int = 100
    c_xsph: float = 0.01

    @property
    def n(self) -> int:
        return len(self.x)

    @property
    def ns(self) -> int:
        return len(self.solid)


def lattice(dims, origin=(0.0, 0.0, 0.0), spacing=1.0) -> np.ndarray:
    """init_chunk_from_grid order: x outer, then y, then z."""
    X, Y, Z = dims
    ix, iy, iz = np.meshgrid(np.arange(X), np.arange(Y), np.arange(Z), indexing="ij")
    idx = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], 1).astype(np.float32)
    p = idx * np.float32(spacing)
    p = p + np.asarray(origin, np.float32)
    return (p + np.float32(spacing * 0.5)).astype(np.float32)


def jitter(x: np.ndarray, amount: float, rng: np.random.Generator) -> np.ndarray:
    return (x + rng.uniform(-amount, amount, x.shape).astype(np.float32)).astype(np.float32)


def value_noise(shape, rng: np.random.Generator, octaves=((8, 1.0), (16, 0.5), (32, 0.25))):
    """Seeded value noise in [0, 1]: bilinear interpolation of random lattices."""
    H, W = shape
    out = np.zeros(shape, np.float64)
    total = 0.0
    for cells, amp in octaves:
        g = rng.random((cells + 1, cells + 1))
        u = np.linspace(0, cells, H, endpoint=False)
        w = np.linspace(0, cells, W, endpoint=False)
        i0, j0 = np.floor(u).astype(int), np.floor(w).astype(int)
        fu, fw = (u - i0)[:, None], (w - j0)[None, :]
        a = g[i0][:, j0]
        b = g[i0 + 1][:, j0]
        c = g[i0][:, j0 + 1]
        d = g[i0 + 1][:, j0 + 1]
        out += amp * (a * (1 - fu) * (1 - fw) + b * fu * (1 - fw) + c * (1 - fu) * fw + d * fu * fw)
        total += amp
    out /= total
    return (out - out.min()) / max(out.max() - out.min(), 1e-12)


def heightmap_solids(size=64, target=50_000, origin=(64, 0, 32), rng=None, max_height=None):
    """Voxelise a seeded heightmap (size x size columns, unit cells) into solid
    particles at voxel centres; heights are scaled so the count is within 1%
    of target.  Returns (solids (ns, 3) float32, heights (size, size))."""
    rng = rng or np.random.default_rng(0)
    noise = value_noise((size, size), rng)
    lo, hi = 0.0, 64.0
    for _ in range(60):
        a = 0.5 * (lo + hi)
        h = np.maximum(1, np.round(1 + a * noise)).astype(int)
        if max_height:
            h = np.minimum(h, max_height)
        if h.sum() < target:
            lo = a
        else:
            hi = a
    h = np.maximum(1, np.round(1 + hi * noise)).astype(int)
    if max_height:
        h = np.minimum(h, max_height)
    pts = []
    for xx in range(size):
        for zz in range(size):
            for yy in range(h[xx, zz]):
                pts.append((xx, yy, zz))
    p = np.asarray(pts, np.float32) + np.asarray(origin, np.float32) + np.float32(0.5)
    return p.astype(np.float32), h


def config0(seed=0) -> Scene:
    """Plain PBF dam break: 10,000 particles.  The stated 20 x 20 x 40 block
    holds 16,000 lattice sites, so the block is 20 x 25 x 20 (10,000) at unit
    spacing from (10, 0, 10) in a 40^3 box; jitter U(-0.05, 0.05)."""
    rng = np.random.default_rng(seed)
    x = jitter(lattice((20, 25, 20), (10, 0, 10)), 0.05, rng)
    return Scene("config0_dam_break_10k", (40, 40, 40), x, dt=1 / 60, iterations=4, steps=100)


def config1(seed=1) -> Scene:
    """262,144 fluid particles (64^3 lattice, jittered) plus ~50k solid
    particles from a seeded 64 x 64 heightmap, box 128 x 64 x 128."""
    rng = np.random.default_rng(seed)
    x = jitter(lattice((64, 64, 64), (0, 0, 0)), 0.05, rng)
    solid, _ = heightmap_solids(64, 50_000, origin=(64, 0, 32), rng=rng, max_height=60)
    return Scene("config1_voxel_solids_262k", (128, 64, 128), x, solid, dt=1 / 60, iterations=4,
                 steps=500)


def config2(seed=2) -> Scene:
    """2,097,152 particles (128^3 lattice, jittered) in a 256 x 128 x 256 box."""
    rng = np.random.default_rng(seed)
    x = jitter(lattice((128, 128, 128), (0, 0, 0)), 0.05, rng)
    return Scene("config2_dam_break_2M", (256, 128, 256), x, dt=1 / 120, iterations=6, steps=200)


def batched_counts(num=512, lo=1024, hi=65536, seed=3) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.round(np.exp(rng.uniform(np.log(lo), np.log(hi), num))).astype(np.int64)


def batched_scene(n: int, rng: np.random.Generator) -> Scene:
    """A cubic-ish block of n particles at unit spacing (lattice sites filled
    layer by layer from the floor) in a box of side 2 * ceil(n^(1/3)) and
    height ceil(n^(1/3)) + 2, jittered by U(-0.05, 0.05)."""
    a = int(np.ceil(n ** (1.0 / 3.0)))
    full = lattice((a, a, a))
    order = np.lexsort((full[:, 2], full[:, 0], full[:, 1]))  # y outer: fill from the floor
    x = jitter(full[order[:n]], 0.05, rng)
    side = max(8, 2 * a)
    return Scene(f"scene_{n}", (side, a + 2, side), x, dt=1 / 60, iterations=4, steps=100)


def config3(seed=3, num=512):
    counts = batched_counts(num, seed=seed)
    rng = np.random.default_rng(seed + 1000)
    return [batched_scene(int(c), rng) for c in counts]


def config4(seed=4, blobs=16, blob=64) -> Scene:
    """16 blobs of 64^3 jittered particles at seeded, non-overlapping centres
    in a 4096 x 256 x 4096 domain (4,194,304 particles)."""
    rng = np.random.default_rng(seed)
    base = lattice((blob, blob, blob))
    placed = []
    parts = []
    while len(placed) < blobs:
        o = np.array([rng.integers(0, 4096 - blob), rng.integers(0, 256 - blob),
                      rng.integers(0, 4096 - blob)], np.float32)
        if any(np.all(np.abs(o - q) < blob + 2) for q in placed):
            continue
        placed.append(o)
        parts.append(jitter(base + o, 0.05, rng))
    x = np.concatenate(parts).astype(np.float32)
    return Scene("config4_precision_4M", (4096, 256, 4096), x, dt=1 / 60, iterations=8, steps=100)
