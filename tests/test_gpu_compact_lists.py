"""Compact neighbour lists (16-byte records: the count, the scene's first
slot and 6 + 8 entries as 16-bit scene offsets; for larger scenes wide
records with the count and 3 + 4 entries as 32-bit slots; longer lists go
on in the column rows) against the column lists: the same entries in the
same order, so every pass sums the same terms in the same order and the
step's fp32 results are bitwise equal; and the cases where the step must
keep column lists."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(sc, p, list_format, unroll=2, xsph_unroll=8, steps=3, solids=None):
    from lustrine_gb300 import PbfSim
    sim = PbfSim(p, sc.n, 0 if solids is None else len(solids))
    sim.upload(sc.x, None, solids)
    sim.set_tuning(128, unroll, 128, xsph_unroll, 1, list_format=list_format)
    sim.step(sc.dt, steps)
    assert sim.status() == 0
    out = sim.download(lambdas=True, density=True)
    fmt = sim.list_format()
    cnt, idx = sim.neighbors()
    sim.close()
    return out, fmt, cnt, idx


def _params(sc, precision, **kw):
    from lustrine_gb300 import pbf_params
    p = pbf_params(*sc.domain, iterations=sc.iterations, c_xsph=sc.c_xsph, precision=precision)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def _assert_same(a, b):
    for u, w in zip(a, b):
        np.testing.assert_array_equal(u, w)


@pytest.mark.parametrize("precision", [0, 2])
def test_compact_lists_give_the_column_bits(precision):
    """Config-0 dam break (10,000 particles): compact lists with 1, 2, 4 and 8
    gathers in flight against column lists, positions, velocities, lambdas,
    densities and the neighbour lists all equal."""
    from lustrine_gb300 import LISTS_COLUMN, LISTS_COMPACT, scenes
    sc = scenes.config0(seed=41)
    ref, fmt, cnt0, idx0 = _run(sc, _params(sc, precision), LISTS_COLUMN)
    assert fmt == "column"
    for unroll in (1, 2, 4, 8):
        got, fmt, cnt, idx = _run(sc, _params(sc, precision), LISTS_COMPACT, unroll, unroll)
        assert fmt == "compact"
        _assert_same(ref, got)
        np.testing.assert_array_equal(cnt0, cnt)
        np.testing.assert_array_equal(idx0, idx)


@pytest.mark.parametrize("grid", ["dense", "hashed"])
@pytest.mark.parametrize("unroll", [1, 2, 4, 8])
@pytest.mark.parametrize("dims,fmt_expected", [((14, 12, 14), "compact"), ((42, 40, 42), "compact_wide")])
def test_compact_overflow_rows(grid, unroll, dims, fmt_expected):
    """A block at spacing 0.6 h: about 18 neighbours a particle, so every list
    fills both records and runs on into the overflow rows (padded with the
    sentinel to the chunk); 2,352 particles take 16-bit entries, 70,560 wide
    records.  On the dense grid (a stencil row's cells walked as one slot
    range) and the hashed grid (each cell's bucket walked on its own) the
    results and lists equal the column lists'."""
    from lustrine_gb300 import LISTS_COLUMN, LISTS_COMPACT, scenes
    from lustrine_gb300._lib import GRID_DENSE, GRID_HASHED
    rng = np.random.default_rng(42)
    x = scenes.jitter(scenes.lattice(dims, (4, 1, 4)) * 0.6, 0.05, rng)
    box = int(np.ceil(0.6 * max(dims))) + 6
    sc = scenes.Scene("dense", (box, box, box), x.astype(np.float32), dt=1 / 60, iterations=4)
    p = _params(sc, 0, grid_mode=GRID_HASHED if grid == "hashed" else GRID_DENSE)
    ref, _, cnt0, idx0 = _run(sc, p, LISTS_COLUMN, unroll, unroll, steps=2)
    got, fmt, cnt, idx = _run(sc, p, LISTS_COMPACT, unroll, unroll, steps=2)
    assert fmt == fmt_expected
    assert (cnt0 > 7).mean() > 0.5  # count includes the particle itself
    _assert_same(ref, got)
    np.testing.assert_array_equal(cnt0, cnt)
    np.testing.assert_array_equal(idx0, idx)


@pytest.mark.parametrize("grid", ["dense", "hashed"])
@pytest.mark.parametrize("max_nbrs", [5, 8, 16])
def test_compact_lists_at_their_capacity(grid, max_nbrs):
    """Lists cut at max_neighbors (5: inside the first record; 8: into the
    second; 16: past both into the overflow rows) on the dense block, on the
    dense and the hashed grid: the overflow status is raised, and results
    (the first lambda sums the dropped entries after the listed ones) and
    the truncated lists equal the column lists'."""
    from lustrine_gb300 import LISTS_COLUMN, LISTS_COMPACT, PbfSim, scenes
    from lustrine_gb300._lib import GRID_DENSE, GRID_HASHED
    rng = np.random.default_rng(45)
    x = scenes.jitter(scenes.lattice((14, 12, 14), (4, 1, 4)) * 0.6, 0.05, rng).astype(np.float32)
    sc = scenes.Scene("dense", (16, 16, 16), x, dt=1 / 60, iterations=4)
    gm = GRID_HASHED if grid == "hashed" else GRID_DENSE
    res = []
    for lf in (LISTS_COLUMN, LISTS_COMPACT):
        sim = PbfSim(_params(sc, 0, max_neighbors=max_nbrs, grid_mode=gm), sc.n)
        sim.upload(sc.x)
        sim.set_tuning(128, 2, 128, 2, 1, list_format=lf)
        sim.step(sc.dt)
        assert sim.status() == 4  # LUSTRINE_ERR_NBR_OVERFLOW: lists truncated
        res.append((sim.download(lambdas=True, density=True), sim.list_format(), sim.neighbors(cap=max_nbrs + 1)))
        sim.close()
    assert res[1][1] == "compact"
    _assert_same(res[0][0], res[1][0])
    _assert_same(res[0][2], res[1][2])


def test_compact_lists_need_counts_below_256():
    """The compact count field holds 8 bits: max_neighbors 256 keeps column lists."""
    from lustrine_gb300 import LISTS_COMPACT, PbfSim, scenes
    sc = scenes.config0(seed=46)
    for cap, want in ((255, "compact"), (256, "column")):
        sim = PbfSim(_params(sc, 0, max_neighbors=cap), sc.n)
        sim.upload(sc.x)
        sim.set_tuning(128, 2, 128, 2, 1, list_format=LISTS_COMPACT)
        sim.step(sc.dt)
        assert sim.status() == 0 and sim.list_format() == want
        sim.close()


@pytest.mark.parametrize("precision", [0, 2])
def test_wide_records_give_the_column_bits(precision):
    """A dam break of 70,560 particles (past the 16-bit entries' 65,535): wide
    records at 1, 2 and 4 gathers in flight against column lists."""
    from lustrine_gb300 import LISTS_COLUMN, LISTS_COMPACT, scenes
    rng = np.random.default_rng(44)
    x = scenes.jitter(scenes.lattice((42, 40, 42)), 0.05, rng)
    sc = scenes.Scene("wide", (84, 44, 84), x, dt=1 / 60, iterations=4)
    ref, fmt, cnt0, idx0 = _run(sc, _params(sc, precision), LISTS_COLUMN)
    assert fmt == "column"
    for unroll in (1, 2, 4):
        got, fmt, cnt, idx = _run(sc, _params(sc, precision), LISTS_COMPACT, unroll, unroll)
        assert fmt == "compact_wide"
        _assert_same(ref, got)
        np.testing.assert_array_equal(cnt0, cnt)
        np.testing.assert_array_equal(idx0, idx)


def test_compact_lists_follow_particles_in_and_out():
    """Sources and sinks change the particle count between steps (the records
    and the sentinel slot n move with it): spawning and despawning the same
    particles in a compact and a column context gives the same bits."""
    from lustrine_gb300 import LISTS_COLUMN, LISTS_COMPACT, PbfSim, scenes
    sc = scenes.config0(seed=49)
    rng = np.random.default_rng(50)
    add = scenes.jitter(scenes.lattice((6, 4, 6), (2, 30, 2)), 0.05, rng)
    res = []
    for lf in (LISTS_COLUMN, LISTS_COMPACT):
        sim = PbfSim(_params(sc, 0), sc.n)
        sim.reserve(sc.n + 2 * len(add))
        sim.upload(sc.x)
        sim.set_tuning(128, 2, 128, 2, 1, list_format=lf)
        sim.step(sc.dt, 2)
        sim.spawn(add)
        sim.step(sc.dt, 2)
        removed = sim.despawn_cells(np.arange(0, 4000, 7, dtype=np.int32))
        sim.step(sc.dt, 2)
        sim.spawn(add + np.float32(1.5))
        sim.step(sc.dt, 2)
        assert sim.status() == 0
        res.append((removed, sim.n, sim.list_format(), sim.download(lambdas=True, density=True)))
        sim.close()
    assert res[1][2] == "compact"
    assert res[0][:2] == res[1][:2]
    _assert_same(res[0][3], res[1][3])


@pytest.mark.parametrize("precision", [0, 2])
def test_compact_batch_equals_column_batch(precision):
    """48 scenes of the batched distribution (the smaller ones, 1,029 to about
    6,000 particles): compact records carry each scene's first slot; the
    batch's results and lists equal the column lists'."""
    from lustrine_gb300 import LISTS_COLUMN, LISTS_COMPACT, PbfSim, pbf_params, scenes
    scs = sorted(scenes.config3(), key=lambda s: s.n)[:48]
    x = np.concatenate([s.x for s in scs])
    res = []
    for lf in (LISTS_COLUMN, LISTS_COMPACT):
        b = PbfSim.batch(pbf_params(8, 8, 8, iterations=4, precision=precision), [s.domain for s in scs],
                         [s.n for s in scs])
        b.upload(x)
        b.set_tuning(128, 4, 128, 4, 1, list_format=lf)
        b.step(scs[0].dt, 3)
        assert b.status() == 0
        res.append((b.download(lambdas=True, density=True), b.list_format(), b.neighbors()))
        b.close()
    assert res[0][1] == "column" and res[1][1] == "compact"
    _assert_same(res[0][0], res[1][0])
    _assert_same(res[0][2], res[1][2])


def test_compact_lists_only_where_they_apply():
    """Scenes of 65,535 particles take 16-bit entries, 65,536 wide records
    (one 16-bit value is kept for the sentinel); static particles, the
    cell-relative mixed form (cell codes in the entries), two particles per
    thread, an s_corr exponent that is not an integer in [0, 32] and the
    reference's step keep column lists."""
    from lustrine_gb300 import (LISTS_COMPACT, MODE_REFERENCE, PRECISION_MIXED, PbfSim, pbf_params,
                                reference_params, scenes)
    rng = np.random.default_rng(43)
    big = scenes.jitter(scenes.lattice((64, 17, 64)), 0.05, rng)[:65536]

    def fmt_of(p, x, solids=None, ppt=1):
        sim = PbfSim(p, len(x), 0 if solids is None else len(solids))
        sim.upload(x, None, solids)
        sim.set_tuning(128, 2, 128, 2, ppt, list_format=LISTS_COMPACT)
        sim.step(1 / 60)
        assert sim.status() == 0
        f = sim.list_format()
        sim.close()
        return f

    assert fmt_of(pbf_params(130, 40, 130), big[:65535]) == "compact"
    assert fmt_of(pbf_params(130, 40, 130), big) == "compact_wide"
    small = big[:4000]
    assert fmt_of(pbf_params(130, 40, 130, precision=PRECISION_MIXED), small) == "column"
    assert fmt_of(pbf_params(130, 40, 130), small, ppt=2) == "column"
    assert fmt_of(pbf_params(130, 40, 130, s_corr_n=2.5), small) == "column"
    assert fmt_of(pbf_params(130, 40, 130, s_corr_n=3.0), small) == "compact"
    solid, _ = scenes.heightmap_solids(16, 300, origin=(0, 0, 0), rng=rng, max_height=2)
    assert fmt_of(pbf_params(130, 40, 130), small, solids=solid) == "column"
    rp = reference_params(130, 40, 130, 0.5, 2.0)
    assert fmt_of(rp, small) == "column"
    # a batch with one scene past the 16-bit limit takes wide records for all
    b = PbfSim.batch(pbf_params(8, 8, 8, iterations=2), [(130, 40, 130), (40, 40, 40)], [65536, 1000])
    b.upload(np.concatenate([big, scenes.jitter(scenes.lattice((10, 10, 10), (5, 0, 5)), 0.05, rng)]))
    b.step(1 / 60)
    assert b.status() == 0 and b.list_format() == "compact_wide"
    b.close()
