"""Particles entering and leaving a scene: spawn (sources) and cell despawn
(sinks, Lustrine.cpp:745-861) on the device, and the reference's source/sink
entry points driving them.

- spawn appends particles as caller indices n, n+1, ... and the state of the
  others is untouched; the capacity bounds it;
- despawn follows the reference's removal sequence exactly: the binned
  particles of the listed cells (in list order, ascending index within a
  cell) each take the data of the current last particle -- restated here on
  the downloaded arrays, with the binning of a reference-mode step restated in
  float32 (its kernels do no FMA contraction);
- the wrapper's simulate (sources before the step, sinks after, timers) is
  restated in float32 numpy over the context API and must give the same
  positions frame by frame."""
import numpy as np
import pytest

from conftest import golden, phys_params
from test_gpu_queries import _box_cells, _cells, _predicted_ref

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1])
def test_spawn_appends_and_capacity_bounds(precision):
    from lustrine_gb300 import LustrineError, PbfSim, pbf_params, scenes
    rng = np.random.default_rng(2)
    x = scenes.jitter(scenes.lattice((8, 6, 8), (4, 2, 4)), 0.05, rng)
    n = len(x)
    sim = PbfSim(pbf_params(24, 20, 24, precision=precision), n)
    sim.reserve(n + 100)
    sim.upload(x)
    with pytest.raises(LustrineError):
        sim.reserve(n + 200)  # after the first upload
    sim.step(1 / 60, 2)
    x1, v1, _, _ = sim.download()
    add = scenes.lattice((4, 3, 5), (15, 12, 15)).astype(np.float32)
    vadd = rng.normal(size=add.shape).astype(np.float32)
    sim.spawn(add, vadd)
    assert sim.n == n + len(add)
    x2, v2, _, _ = sim.download()
    np.testing.assert_array_equal(x2[:n], x1)
    np.testing.assert_array_equal(v2[:n], v1)
    np.testing.assert_array_equal(x2[n:], add)
    np.testing.assert_array_equal(v2[n:], vadd)
    sim.step(1 / 60, 3)
    assert sim.status() == 0
    assert sim.query_cell_count((0, 0, 0), (24, 20, 24)) == n + len(add)
    with pytest.raises(LustrineError):
        sim.spawn(np.zeros((41, 3), np.float32) + 5.0)  # 60 + 41 > 100 of room
    sim.spawn(np.zeros((0, 3), np.float32))
    sim.close()


def _swap_remove(x, v, evict):
    x, v = x.copy(), v.copy()
    end = len(x)
    for e in evict:
        x[e] = x[end - 1]
        v[e] = v[end - 1]
        end -= 1
    return x[:end], v[:end]


def test_despawn_matches_the_reference_removal_sequence():
    from lustrine_gb300 import PbfSim, reference_params
    g = golden("ref_solids_2step.npz")
    n, ns = len(g["x0"]), len(g["solid"])
    domain = tuple(int(a) for a in g["domain"])
    p = phys_params(reference_params(*domain))
    sim = PbfSim(p, n, ns)
    sim.upload(g["x0"], g["v0"], g["solid"])
    dt = float(g["dt"])
    sim.step(dt)
    x1, v1, _, _ = sim.download()
    grid = [int(d / p.cell_size) + 1 for d in domain]
    fc = _cells(_predicted_ref(g["x0"], g["v0"], p, dt), p.cell_size, grid)
    cid = fc[:, 1] * grid[0] * grid[2] + fc[:, 0] * grid[2] + fc[:, 2]
    occupied = np.unique(cid)
    # a block of occupied cells, a repeated cell, and the cells of the last
    # particles (evictions that reach the tail move and drop particles in the
    # reference's way)
    cells = list(occupied[5:40]) + [occupied[7]] + [int(cid[n - 1]), int(cid[n - 3])]
    evict = []
    for c in cells:
        evict += sorted(np.nonzero(cid == c)[0].tolist())
    ex, ev = _swap_remove(x1, v1, evict)
    removed = sim.despawn_cells(np.array(cells, np.int32))
    assert removed == n - len(ex) and sim.n == len(ex)
    x2, v2, _, _ = sim.download()
    np.testing.assert_array_equal(x2, ex)
    np.testing.assert_array_equal(v2, ev)
    # the cell table follows the survivors
    assert sim.query_cell_count((0, 0, 0), domain, False) == len(ex)
    assert sim.query_cell_count((0, 0, 0), domain, True) == len(ex) + ns
    sim.step(dt, 2)
    assert sim.status() == 0
    # a cell nothing is binned in: no-op
    top = (grid[1] - 1) * grid[0] * grid[2] + (grid[0] - 1) * grid[2] + grid[2] - 1
    assert sim.despawn_cells(np.array([top], np.int32)) == 0 and sim.n == len(ex)
    sim.close()


def _pattern_positions(X, Y, Z, position, d):
    return np.array([(np.float32(x) * np.float32(d) + np.float32(position[0]) + np.float32(d / 2),
                      np.float32(y) * np.float32(d) + np.float32(position[1]) + np.float32(d / 2),
                      np.float32(z) * np.float32(d) + np.float32(position[2]) + np.float32(d / 2))
                     for x in range(X) for y in range(Y) for z in range(Z)], np.float32)


def test_wrapper_sources_and_sinks_match_a_restatement():
    from lustrine_gb300 import PbfSim, reference_params
    from lustrine_gb300 import wrapper as W
    from lustrine_gb300._lib import SimulationParameters
    from test_gpu_queries import _box_solid_positions
    f = np.float32
    prm = SimulationParameters(20, 20, 20, 0.5, 1.0)
    sand = W.init_grid_box(prm, 4, 4, 4, (8.0, 6.0, 8.0), type_=1)
    floor = W.init_grid_box(prm, 20, 1, 20, (0.0, 0.0, 0.0), type_=0)
    pattern = W.init_grid_box(prm, 2, 1, 2, (10.0, 14.0, 10.0), type_=1)
    try:
        W.init_simulation_extra_parameters(prm, [sand], [floor], 1, 2.0)
        assert W.last_status() == 0
        W.set_simulate_function(2)  # the fluid step (simulate_sand follows init)
        assert W.last_status() == 0
        n0 = W.get_num_sand_particles()
        src = W.add_particle_source(pattern, (0.0, -1.0, 0.0), 0.03, 12)
        snk = W.add_particle_sink((7, 5, 7), (10, 7.5, 10), 0.0)  # the block's lower corner
        assert (src, snk) == (0, 0) and W.last_status() == 0
        # the same scene through the context API, with the frame logic restated
        p = reference_params(20, 20, 20, 0.5, 2.0)
        x0 = W.simulation_bind_positions_copy()
        solid = _box_solid_positions(20, 1, 20, (0.0, 0.0, 0.0), 1.0)
        sim = PbfSim(p, n0, len(solid))
        sim.reserve(n0 + 100)
        sim.upload(x0, None, solid)
        pat = _pattern_positions(2, 1, 2, (10.0, 14.0, 10.0), 1.0)
        d = np.array([0.0, -1.0, 0.0], np.float32)
        d = d / np.float32(np.sqrt(np.float32(d @ d)))
        grid = [21, 21, 21]
        r = _box_cells((7, 5, 7), (10, 7.5, 10), (20, 20, 20), p.cell_size)
        sink_cells = np.array([y * grid[0] * grid[2] + x * grid[2] + z
                               for y in range(r[1][0], r[1][1] + 1)
                               for x in range(r[0][0], r[0][1] + 1)
                               for z in range(r[2][0], r[2][1] + 1)], np.int32)
        timer, total_time, spawned, sink_timer = f(0), f(0), 0, f(0)
        dt = 1 / 60
        for frame in range(8):
            timer = f(timer + f(0.016))
            if spawned < 12 and timer >= f(0.03):
                freq = f(0.03)
                offset = f(freq - np.fmod(total_time, freq))
                speed = f(f(f(1.0) * f(1.0)) / freq)
                xs = (pat + d * offset).astype(np.float32)
                vs = np.tile(d * speed, (len(pat), 1)).astype(np.float32)
                vs[len(pat) // 2] += f(0.001)
                sim.spawn(xs, vs)
                spawned += len(pat)
                timer = f(0)
            sim.step(dt)
            if sink_timer >= f(0.0):
                sim.despawn_cells(sink_cells)
            sink_timer = f(sink_timer + f(dt))
            total_time = f(total_time + f(0.016))
            W.simulate(dt, False, False)
            assert W.last_status() == 0
            assert W.get_num_sand_particles() == sim.n
            np.testing.assert_array_equal(W.simulation_bind_positions_copy(), sim.positions())
        assert W.get_source_spawned(0) == 12 == spawned
        assert W.get_num_sand_particles() < n0 + spawned  # the sink removed particles
        assert W.get_sink_despawned(0) == 0  # the reference never counts it
        W.set_source_state(0, False)
        W.set_sink_state(0, False)
        assert W.last_status() == 0
        W.get_source_spawned(5)
        assert W.last_status() != 0
        sim.close()
    finally:
        W.cleanup_simulation()
        for g_ in (sand, floor, pattern):
            W.free_grid(g_)
