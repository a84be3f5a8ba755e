"""Sand mode (simulate_sand, Simulate.cpp:156-325) on the GPU against the
reference's own five steps (golden fixture) and against the oracle's
restatement on larger seeded scenes.  Everything is compared bit for bit:
positions, velocities, attract flags and the neighbour lists in the
reference's order (the reference also lists each particle twice in its own
list; the GPU leaves it out and the substeps skip it)."""
import numpy as np
import pytest

from conftest import golden, phys_params

pytestmark = pytest.mark.gpu


def _params(domain, mass=1.0, gravity=-9.81, max_neighbors=96, use_graph=True):
    from lustrine_gb300 import sand_params
    return sand_params(*domain, mass=mass, gravity=gravity, max_neighbors=max_neighbors,
                       use_graph=use_graph)


def _strip_self(cnt, idx):
    """Reference-order lists without the particle's own entries."""
    out = []
    for i in range(len(cnt)):
        row = idx[i, :cnt[i]]
        out.append(row[row != i])
    return out


def _gpu_lists(sim):
    cnt, idx = sim.neighbors()
    return [idx[i, :cnt[i]] for i in range(len(cnt))]


def test_sand_matches_reference_five_steps():
    """The reference's fixture: no flags, attract twice, blow, no flags."""
    from lustrine_gb300 import PbfSim
    g = golden("ref_sand_steps.npz")
    n, ns = len(g["x0"]), len(g["solid"])
    sim = PbfSim(_params(tuple(int(a) for a in g["domain"])), n, ns)
    sim.upload(g["x0"], g["v0"], g["solid"])
    for k in range(len(g["attract"])):
        s = k + 1
        sim.set_sand_controls(player=g["player"][k], attract=bool(g["attract"][k]), blow=bool(g["blow"][k]),
                              diameter=float(g["diameter"]))
        sim.step(float(g["dt"]))
        x, v, _, _ = sim.download()
        assert np.array_equal(x, g[f"x{s}"]), f"step {s}: x"
        assert np.array_equal(v, g[f"v{s}"]), f"step {s}: v"
        assert np.array_equal(sim.attracted(), g[f"att{s}"]), f"step {s}: attracted"
        off, flat = g[f"nbr_off{s}"], g[f"nbr{s}"]
        ref = [flat[off[i]:off[i + 1]] for i in range(n)]
        ref = [r[r != i] for i, r in enumerate(ref)]
        got = _gpu_lists(sim)
        assert all(np.array_equal(a, b) for a, b in zip(got, ref)), f"step {s}: lists"
    assert sim.status() == 0
    sim.close()


def _pile(rng, block, origin, domain):
    """A jittered block of sand at unit spacing above a seeded heightmap of
    static particles (voxel centres)."""
    from lustrine_gb300 import scenes
    x = scenes.jitter(scenes.lattice(block, origin), 0.05, rng)
    X, _, Z = domain
    H = rng.integers(1, 4, size=(X, Z))
    sx, sz = np.meshgrid(np.arange(X), np.arange(Z), indexing="ij")
    solid = [np.stack([sx.ravel() + 0.5, np.full(X * Z, y + 0.5), sz.ravel() + 0.5], 1)[H.ravel() > y]
             for y in range(3)]
    return x.astype(np.float32), np.concatenate(solid).astype(np.float32)


@pytest.mark.parametrize("use_graph", [True, False])
def test_sand_matches_oracle_with_controls(orc, use_graph):
    """20,000 sand particles over 1,500+ static ones, six steps with the
    player attracting, then blowing, then neither: GPU == oracle bit for bit."""
    from lustrine_gb300 import PbfSim
    rng = np.random.default_rng(21)
    domain = (48, 40, 48)
    x, solid = _pile(rng, (25, 32, 25), (12, 4, 12), domain)
    n, ns = len(x), len(solid)
    sim = PbfSim(_params(domain, use_graph=use_graph), n, ns)
    sim.upload(x, None, solid)
    p = phys_params(orc.reference_params(*domain))
    xo, vo, ao = x.copy(), np.zeros_like(x), np.zeros(n, np.int32)
    plan = [dict(), dict(attract=True, player=(24.0, 20.0, 24.0)), dict(attract=True, player=(26.0, 18.0, 24.0)),
            dict(blow=True, player=(20.0, 10.0, 20.0)), dict(blow=True, attract=True, player=(30.0, 8.0, 30.0)),
            dict()]
    prev = False
    att_seen = 0
    for c in plan:
        ctl = orc.sand_controls(prev_attract=prev, diameter=1.0, **c)
        sim.set_sand_controls(player=ctl.player_position[:], attract=bool(ctl.attract_flag),
                              blow=bool(ctl.blow_flag), diameter=1.0)
        sim.step(1.0 / 60.0)
        o = orc.sand_step(p, ctl, np.float32(1.0 / 60.0), xo, vo, ao, solid=solid, cap=96)
        xo, vo, ao = o["x"], o["v"], o["attracted"]
        att_seen = max(att_seen, int(ao.sum()))
        prev = bool(c.get("attract", False))
        x, v, _, _ = sim.download()
        assert np.array_equal(x, xo) and np.array_equal(v, vo)
        assert np.array_equal(sim.attracted(), ao)
        ref = _strip_self(o["nbr_count"], o["nbr_idx"])
        got = _gpu_lists(sim)
        assert all(np.array_equal(a, b) for a, b in zip(got, ref))
    assert att_seen > 0, "the plan must attract some particles"
    assert sim.status() == 0
    sim.close()


def test_sand_full_size_pile_one_step_exact(orc):
    """262,144 sand particles (64^3 block) over a 128 x 128 heightmap: one
    step equal to the oracle, and a second step keeps every particle in the
    box with finite velocities."""
    from lustrine_gb300 import PbfSim
    rng = np.random.default_rng(5)
    domain = (128, 80, 128)
    x, solid = _pile(rng, (64, 64, 64), (32, 4, 32), domain)
    n, ns = len(x), len(solid)
    sim = PbfSim(_params(domain), n, ns)
    sim.upload(x, None, solid)
    sim.step(1.0 / 60.0)
    p = phys_params(orc.reference_params(*domain))
    o = orc.sand_step(p, orc.sand_controls(diameter=1.0), np.float32(1.0 / 60.0), x, np.zeros_like(x), None,
                      solid=solid, cap=96)
    xg, vg, _, _ = sim.download()
    assert np.array_equal(xg, o["x"]) and np.array_equal(vg, o["v"])
    sim.step(1.0 / 60.0)
    xg, vg, _, _ = sim.download()
    assert np.isfinite(vg).all()
    assert (xg >= 0.5).all() and (xg[:, 0] <= 127.5).all() and (xg[:, 1] <= 79.5).all()
    assert sim.status() == 0
    sim.close()


def test_sand_without_static_particles_and_empty():
    from lustrine_gb300 import PbfSim
    rng = np.random.default_rng(3)
    from lustrine_gb300 import scenes
    x = scenes.jitter(scenes.lattice((8, 8, 8), (4, 0, 4)), 0.05, rng)
    sim = PbfSim(_params((16, 16, 16)), len(x), 0)
    sim.upload(x)
    sim.step(1.0 / 60.0, 3)
    xg, vg, _, _ = sim.download()
    assert np.isfinite(xg).all() and sim.status() == 0
    assert sim.launches_per_step() == 10
    sim.close()
    empty = PbfSim(_params((8, 8, 8)), 0, 0)
    empty.upload(np.zeros((0, 3), np.float32))
    empty.step(1.0 / 60.0)
    assert empty.status() == 0
    empty.close()


def test_wrapper_runs_simulate_sand_after_init(orc):
    """The reference's C entry points: init_simulation_extra_parameters leaves
    simulate_sand selected (Lustrine.cpp:312); simulate(dt, attract, blow)
    passes its flags, simulate_no_flags keeps them; positions come back in
    the reference's order (re-sorted by cell every step)."""
    from lustrine_gb300 import wrapper as W
    from lustrine_gb300._lib import SimulationParameters
    from test_gpu_queries import _box_solid_positions
    prm = SimulationParameters(20, 20, 20, 0.5, 1.0)
    sand = W.init_grid_box(prm, 6, 5, 6, (5.0, 3.0, 5.0), type_=1)
    floor = W.init_grid_box(prm, 20, 1, 20, (0.0, 0.0, 0.0), type_=0)
    try:
        W.init_simulation_extra_parameters(prm, [sand], [floor], 1, 2.0)
        assert W.last_status() == 0
        x = W.simulation_bind_positions_copy()
        solid = _box_solid_positions(20, 1, 20, (0.0, 0.0, 0.0), 1.0)
        p = orc.reference_params(20, 20, 20, 0.5, 2.0)  # mass 5, gravity -10 (Simulation.hpp:157-171)
        v, att = np.zeros_like(x), np.zeros(len(x), np.int32)
        W.set_player_position((8.0, 5.0, 8.0))
        prev, seen = False, 0
        for flags in ((False, False), (True, False), None, (False, True), (False, False)):
            if flags is None:  # the previous call's flags stay
                W.simulate_no_flags(1 / 60)
                flags = last
            else:
                W.simulate(1 / 60, *flags)
            assert W.last_status() == 0
            ctl = orc.sand_controls(player=(8.0, 5.0, 8.0), attract=flags[0], blow=flags[1], prev_attract=prev,
                                    diameter=1.0)
            o = orc.sand_step(p, ctl, np.float32(1 / 60), x, v, att, solid=solid, cap=96)
            x, v, att = o["x"], o["v"], o["attracted"]
            prev, last = flags[0], flags
            seen = max(seen, int(att.sum()))
            assert np.array_equal(W.simulation_bind_positions_copy(), x)
        assert seen > 0, "the player must attract some particles"
        W.set_simulate_function(1)  # simulate_sand_v3 is not provided
        assert W.last_status() != 0
        W.set_simulate_function(0)
        assert W.last_status() == 0
    finally:
        W.cleanup_simulation()
        W.free_grid(sand)
        W.free_grid(floor)


def test_sand_sources_and_sinks_match_oracle(orc):
    """Spawned blocks and a sink on the sand step: the context's spawn,
    step and cell despawn against the oracle's step with the reference's
    spawn (append) and swap-remove eviction (Lustrine.cpp:768-834) of the
    sand particles the step binned in the sink cells."""
    from lustrine_gb300 import PbfSim, scenes
    rng = np.random.default_rng(8)
    domain = (24, 24, 24)
    x, solid = _pile(rng, (6, 6, 6), (9, 4, 9), domain)
    n0 = len(x)
    sim = PbfSim(_params(domain), n0, len(solid))
    sim.reserve(n0 + 64)
    sim.upload(x, None, solid)
    p = phys_params(orc.reference_params(*domain))
    g = [int(a) for a in p.grid]
    sink = np.array([y * g[0] * g[2] + xx * g[2] + z for y in range(3, 6) for xx in range(8, 12)
                     for z in range(8, 12)], np.int32)
    pat = scenes.lattice((2, 1, 2), (11.0, 16.0, 11.0)).astype(np.float32)
    xo, vo, ao = x.copy(), np.zeros_like(x), np.zeros(n0, np.int32)
    ctl = orc.sand_controls(diameter=1.0)
    dt = np.float32(1 / 60)
    for frame in range(10):
        if frame % 3 == 1:
            vs = np.tile(np.array([0.0, -2.0, 0.0], np.float32), (len(pat), 1))
            sim.spawn(pat, vs)
            xo, vo = np.concatenate([xo, pat]), np.concatenate([vo, vs])
            ao = np.concatenate([ao, np.zeros(len(pat), np.int32)])
        sim.step(float(dt))
        o = orc.sand_step(p, ctl, dt, xo, vo, ao, solid=solid, cap=96)
        xo, vo, ao = o["x"].copy(), o["v"].copy(), o["attracted"].copy()
        if frame % 2 == 0:
            removed = sim.despawn_cells(sink)
            keys = ((np.trunc(o["xs"][:, 1] / p.cell_size).astype(np.int64) * g[0] * g[2])
                    + np.trunc(o["xs"][:, 0] / p.cell_size).astype(np.int64) * g[2]
                    + np.trunc(o["xs"][:, 2] / p.cell_size).astype(np.int64))
            evict = [i for c in sink for i in np.nonzero(keys == c)[0]]
            end = len(xo)
            for e in evict:  # Lustrine.cpp:824-832
                xo[e], vo[e], ao[e] = xo[end - 1], vo[end - 1], ao[end - 1]
                end -= 1
            xo, vo, ao = xo[:end], vo[:end], ao[:end]
            assert removed == len(evict)
        xg, vg, _, _ = sim.download()
        assert len(xg) == len(xo)
        assert np.array_equal(xg, xo) and np.array_equal(vg, vo)
        assert np.array_equal(sim.attracted(), ao)
    assert sim.n < n0 + 3 * len(pat)  # the sink removed particles
    assert sim.status() == 0
    sim.close()


def test_wrapper_sand_on_a_vox_floor(orc):
    """A MagicaVoxel model (tests/golden/vox/box.vox) as the static grid of a
    wrapper simulation: its occupied cells become the static particles
    (init_chunk_from_grid order, stored from the end backwards) and the sand
    step over them equals the oracle's."""
    import os
    from conftest import GOLDEN
    from lustrine_gb300 import wrapper as W
    from lustrine_gb300._lib import SimulationParameters
    prm = SimulationParameters(20, 20, 20, 0.5, 1.0)
    floor = W.init_grid_magikavoxel(os.path.join(GOLDEN, "vox", "box.vox"), (6.0, 0.0, 6.0))
    sand = W.init_grid_box(prm, 4, 4, 4, (6.0, 4.0, 6.0), type_=1)
    try:
        cells, _ = W.grid_arrays(floor)
        W.init_simulation_extra_parameters(prm, [sand], [floor], 1, 2.0)
        assert W.last_status() == 0
        solid = np.array([(x + 6.5, y + 0.5, z + 6.5) for x in range(cells.shape[0]) for y in range(cells.shape[1])
                          for z in range(cells.shape[2]) if cells[x, y, z] != 0], np.float32)[::-1]
        x = W.simulation_bind_positions_copy()
        v, att = np.zeros_like(x), np.zeros(len(x), np.int32)
        p = orc.reference_params(20, 20, 20, 0.5, 2.0)
        for _ in range(6):
            W.simulate(1 / 60, False, False)
            assert W.last_status() == 0
            o = orc.sand_step(p, orc.sand_controls(diameter=1.0), np.float32(1 / 60), x, v, att, solid=solid, cap=96)
            x, v, att = o["x"], o["v"], o["attracted"]
            assert np.array_equal(W.simulation_bind_positions_copy(), x)
        assert (o["nbr_idx"] >= len(x)).any(), "the sand must reach the voxel floor"
    finally:
        W.cleanup_simulation()
        W.free_grid(floor)
        W.free_grid(sand)


def test_mode_switch_into_sand_clears_attract_flags():
    """The fluid steps re-sort particles without the sand flags: switching
    from a fluid step back to sand starts with cleared flags, and the
    context keeps stepping in every mode it is switched to."""
    from lustrine_gb300 import MODE_PBF, MODE_REFERENCE, MODE_SAND, PbfSim, scenes
    rng = np.random.default_rng(9)
    x = scenes.jitter(scenes.lattice((8, 8, 8), (4, 2, 4)), 0.05, rng)
    p = _params((16, 16, 16))
    sim = PbfSim(p, len(x), 0)
    sim.upload(x)
    sim.set_attracted(np.ones(len(x), np.int32))
    sim.step(1 / 60)
    assert sim.attracted().sum() == len(x)  # no attraction in play: the flags stay
    for mode in (MODE_REFERENCE, MODE_PBF, MODE_SAND):
        q = sim.params
        q.mode = mode
        if mode == MODE_PBF:
            q.iterations = 2
        sim.set_params(q)
        sim.step(1 / 60, 2)
        assert sim.status() == 0
    assert sim.attracted().sum() == 0
    sim.close()
