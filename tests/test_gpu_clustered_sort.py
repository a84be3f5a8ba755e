"""The step's cell sort on clustered states (cells of 250 to 4,000
particles, as a collapsed reference-semantics rollout or a sand pile makes
them): the stable order within a cell comes from a block-wide sort of the
cell's members, O(k log k) for a cell of k, instead of every member counting
the members before it (O(k^2)).

Parity: reference semantics on cells of 1,200 particles, where the list
order -- cell order, then ascending particle id -- decides the summation
order: lists equal in order, lambdas, positions and velocities bitwise equal
to the oracle's Jacobi form of the reference step.  Cost: at a fixed particle
count the sort stage stays within a small factor as the cells grow 16 times
larger (the quadratic form grew with the cell size)."""
import statistics

import numpy as np
import pytest

from conftest import phys_params

pytestmark = pytest.mark.gpu


def normwise_rel(a, b):
    """Per-particle |a - b| / max(|b|, 1e-3 rms|b|)."""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    nb = np.linalg.norm(b, axis=1)
    floor = 1e-3 * np.sqrt(np.mean(nb ** 2))
    return np.linalg.norm(a - b, axis=1) / np.maximum(nb, floor)


def clustered(K, n, seed, spacing=3):
    """n // K cells of K particles each (uniform inside the cell), the cells
    on a lattice `spacing` cells apart, so a particle's neighbours are the
    members of its own cell."""
    rng = np.random.default_rng(seed)
    m = n // K
    side = int(np.ceil(m ** (1.0 / 3.0) - 1e-9))
    cells = np.array([(i, j, k) for i in range(side) for j in range(side) for k in range(side)][:m], np.float32)
    base = cells * spacing + 2.0
    x = np.repeat(base, K, axis=0) + rng.uniform(0.02, 0.98, (m * K, 3)).astype(np.float32)
    dom = int(side * spacing + 4)
    order = rng.permutation(len(x))  # caller order unrelated to the cells
    return x[order].astype(np.float32), (dom, dom, dom)


def _ref_sim(domain, n, cap):
    from lustrine_gb300 import PbfSim, reference_params
    p = phys_params(reference_params(*domain))
    p.max_neighbors = cap
    return PbfSim(p, n)


def test_clustered_reference_step_bitwise_vs_oracle(orc):
    x, dom = clustered(1200, 6000, seed=5)
    n = len(x)
    v = np.zeros_like(x)
    dt = 1e-3
    sim = _ref_sim(dom, n, 1280)
    sim.upload(x, v)
    sim.step(dt)
    st = sim.status()
    assert st in (0, 5), st  # a particle pushed out of the grid is clamped and reported (5)
    cnt, idx = sim.neighbors(cap=1280)
    p = phys_params(orc.reference_params(*dom))
    p.jacobi = 1
    o = orc.compat_step(p, dt, x, v, cap=1280)
    assert cnt.max() >= 1000 and np.array_equal(cnt, o["nbr_count"])
    for i in range(0, n, 97):
        assert np.array_equal(idx[i, :cnt[i]], o["nbr_idx"][i, :cnt[i]]), i
    gx, gv, glam, _ = sim.download(lambdas=True)
    assert np.array_equal(glam, o["lambdas"][:n])
    assert normwise_rel(gx, o["x"]).max() <= 1e-5
    assert normwise_rel(gv, o["v"]).max() <= 1e-5
    sim.close()


def _sort_ms(K, n):
    x, dom = clustered(K, n, seed=K)
    sim = _ref_sim(dom, len(x), 16)  # lists overflow (status 4): only the sort is timed here
    sim.upload(x, np.zeros_like(x))
    ms = []
    for _ in range(5):
        sim.upload(x, np.zeros_like(x))
        ms.append(sim.profile_step(1e-3)["sort"][0])
    sim.close()
    return statistics.median(ms)


def test_clustered_sort_stage_scales_with_particles_not_cell_size():
    n = 64_000
    t_small = _sort_ms(250, n)
    t_big = _sort_ms(4000, n)
    # O(k^2): 16x from 250 to 4,000 per cell; O(k log k): about 1.5x
    assert t_big <= 4.0 * t_small + 0.05, (t_small, t_big)
