"""Cell-count query (Lustrine::query_cell_num_particles, Lustrine.cpp:864-914)
on the GPU cell table, and the reference's wrapper entry points driving the
reference-mode step.

The query counts the particles the last step binned in the cells of a box:
fluid at the step's predicted positions, solids at theirs, corners clamped to
[cell/2, domain - cell/2] and truncated.  In reference mode the prediction is
restated here in float32 (the reference-mode kernels do no FMA contraction),
so the expected counts are exact."""
import numpy as np
import pytest

from conftest import golden, phys_params

pytestmark = pytest.mark.gpu


def _box_cells(lo, hi, domain, cell):
    """Cell index ranges of a query box, as get_cell_indices forms them."""
    f = np.float32
    out = []
    for a in range(3):
        lo_b = f(np.float64(cell) * 0.5)
        hi_b = f(np.float64(f(domain[a])) - np.float64(cell) * 0.5)
        i0 = int(np.trunc(f(min(max(f(lo[a]), lo_b), hi_b)) / f(cell)))
        i1 = int(np.trunc(f(min(max(f(hi[a]), lo_b), hi_b)) / f(cell)))
        out.append((i0, i1))
    return out


def _cells(pos, cell, grid):
    c = np.trunc(pos.astype(np.float32) / np.float32(cell)).astype(np.int64)
    return np.clip(c, 0, np.asarray(grid) - 1)


def _count(cells, ranges):
    m = np.ones(len(cells), bool)
    for a, (i0, i1) in enumerate(ranges):
        m &= (cells[:, a] >= i0) & (cells[:, a] <= i1)
    return int(m.sum())


def _predicted_ref(x, v, p, dt):
    """Reference prediction (Simulate.cpp:31-51) in float32."""
    f = np.float32
    dtc = f(min(max(dt, 0.001), 0.01))
    gm = np.array(p.gravity[:], np.float32) * f(p.mass)
    v1 = v.astype(np.float32) + gm * dtc
    return x.astype(np.float32) + v1 * dtc


def _boxes(domain, rng, k=12):
    out = [((0, 0, 0), domain), ((-5, -5, -5), (1e6, 1e6, 1e6))]
    for _ in range(k):
        a = rng.uniform(0, np.array(domain, float))
        b = rng.uniform(0, np.array(domain, float))
        out.append((tuple(np.minimum(a, b)), tuple(np.maximum(a, b))))
    return out


def test_query_reference_mode_matches_binning():
    from lustrine_gb300 import PbfSim, reference_params
    g = golden("ref_solids_2step.npz")
    n, ns = len(g["x0"]), len(g["solid"])
    domain = tuple(int(a) for a in g["domain"])
    p = phys_params(reference_params(*domain))
    sim = PbfSim(p, n, ns)
    sim.upload(g["x0"], g["v0"], g["solid"])
    assert sim.query_cell_count((0, 0, 0), domain, True) == 0  # no step yet: empty table
    sim.step(float(g["dt"]))
    assert sim.status() == 0
    grid = [int(d / p.cell_size) + 1 for d in domain]
    fc = _cells(_predicted_ref(g["x0"], g["v0"], p, float(g["dt"])), p.cell_size, grid)
    sc = _cells(g["solid"], p.cell_size, grid)
    rng = np.random.default_rng(5)
    for lo, hi in _boxes(domain, rng):
        r = _box_cells(lo, hi, domain, p.cell_size)
        assert sim.query_cell_count(lo, hi, False) == _count(fc, r), (lo, hi)
        assert sim.query_cell_count(lo, hi, True) == _count(fc, r) + _count(sc, r), (lo, hi)
    assert sim.query_cell_count((0, 0, 0), domain, False) == n
    assert sim.query_cell_count((0, 0, 0), domain, True) == n + ns
    # min above max on an axis: nothing, as the reference's loops
    assert sim.query_cell_count((10, 0, 0), (2, 20, 20), True) == 0
    sim.close()


@pytest.mark.parametrize("grid_mode", [1, 2])
def test_query_pbf_partition_and_totals(grid_mode):
    """PBF mode, dense and hashed grids: the counts of boxes that partition
    the grid's cells add up to the totals."""
    from lustrine_gb300 import PbfSim, pbf_params, scenes
    rng = np.random.default_rng(8)
    x = scenes.jitter(scenes.lattice((12, 10, 12), (6, 4, 6)), 0.05, rng)
    solid, _ = scenes.heightmap_solids(24, 1500, origin=(0, 0, 0), rng=rng, max_height=5)
    domain = (24, 20, 24)
    sim = PbfSim(pbf_params(*domain, grid_mode=grid_mode), len(x), len(solid))
    sim.upload(x, None, solid)
    sim.step(1 / 60, 3)
    assert sim.status() == 0
    n, ns = len(x), len(solid)
    assert sim.query_cell_count((0, 0, 0), domain, False) == n
    assert sim.query_cell_count((0, 0, 0), domain, True) == n + ns
    # cell-centre corners split every axis at cell 10 (cells 0-9 and 10-24)
    tot_f = tot_s = 0
    for bx in ((0.5, 9.5), (10.5, 30.0)):
        for by in ((0.5, 9.5), (10.5, 30.0)):
            for bz in ((0.5, 9.5), (10.5, 30.0)):
                lo, hi = (bx[0], by[0], bz[0]), (bx[1], by[1], bz[1])
                f = sim.query_cell_count(lo, hi, False)
                tot_f += f
                tot_s += sim.query_cell_count(lo, hi, True) - f
    assert tot_f == n and tot_s == ns
    sim.close()


def _box_solid_positions(X, Y, Z, position, diam):
    """init_chunk_from_grid order (x, y, z loops), stored from the end backwards."""
    pts = [((x * diam) + position[0] + diam / 2, (y * diam) + position[1] + diam / 2,
            (z * diam) + position[2] + diam / 2)
           for x in range(X) for y in range(Y) for z in range(Z)]
    return np.array(pts[::-1], np.float32)


def test_wrapper_entry_points_drive_reference_mode(orc):
    """init_grid_box + init_simulation_extra_parameters + simulate through the
    reference's C entry points: the particle order of the reference, the
    reference-mode step (against the oracle's Jacobi form), and
    query_cell_num_particles equal to the context's count."""
    from lustrine_gb300 import wrapper as W
    from lustrine_gb300._lib import SimulationParameters
    prm = SimulationParameters(20, 20, 20, 0.5, 1.0)
    sand = W.init_grid_box(prm, 6, 5, 6, (5.0, 3.0, 5.0), type_=1)
    floor = W.init_grid_box(prm, 20, 1, 20, (0.0, 0.0, 0.0), type_=0)
    try:
        data = W.init_simulation_extra_parameters(prm, [sand], [floor], 1, 2.0)
        assert W.last_status() == 0
        W.set_simulate_function(2)  # the fluid step (simulate_sand follows init)
        assert W.last_status() == 0
        n = W.get_num_sand_particles()
        assert n == data.num_sand_particles == 6 * 5 * 6 and data.num_solid_particles == 400
        x0 = W.simulation_bind_positions_copy()
        lattice = [(x + 5.5, y + 3.5, z + 5.5) for x in range(6) for y in range(5) for z in range(6)]
        assert np.array_equal(x0, np.array(lattice, np.float32))
        solid = _box_solid_positions(20, 1, 20, (0.0, 0.0, 0.0), 1.0)
        p = orc.reference_params(20, 20, 20, 0.5, 2.0)
        p.jacobi = 1
        o = dict(x=x0, v=np.zeros_like(x0), lambdas=None)
        dt = 1 / 60
        for _ in range(2):
            W.simulate(dt, False, False)
            assert W.last_status() == 0
            o = orc.compat_step(p, dt, o["x"], o["v"], solid=solid, lambdas=o["lambdas"])
        x = W.simulation_bind_positions_copy()
        assert np.abs(x - o["x"]).max() <= 1e-5 * 20
        ctx = W.global_context()
        for lo, hi in (((0, 0, 0), (20, 20, 20)), ((4, 0, 4), (12, 6, 12)), ((0, 0, 0), (20, 1.2, 20))):
            for inc in (False, True):
                assert W.query_cell_num_particles(lo, hi, inc) == ctx.query_cell_count(lo, hi, inc)
                assert W.last_status() == 0
        assert W.query_cell_num_particles((0, 0, 0), (20, 20, 20), True) == n + 400
        assert W.query_cell_num_particles((0, 0, 0), (20, 20, 20), False) == n
    finally:
        W.cleanup_simulation()
        W.free_grid(sand)
        W.free_grid(floor)
