"""Batched scenes: one context stepping many independent scenes must give
each scene exactly what stepping it alone gives (same kernels, same lists,
same summation order), in both precisions; and the batched mixed-precision
step keeps the density within 1e-4 of the FP64 oracle (the equal-error
condition of the batched / plain comparison)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scenes():
    from lustrine_gb300 import scenes
    rng = np.random.default_rng(41)
    out = [scenes.batched_scene(int(n), rng) for n in (1024, 3000, 777, 5000)]
    # one scene with solids under the block
    solid, _ = scenes.heightmap_solids(16, 600, origin=(0, 0, 0), rng=rng, max_height=3)
    x = scenes.jitter(scenes.lattice((8, 8, 8), (4, 3, 4)), 0.05, rng)
    out.append(scenes.Scene("solids", (16, 14, 16), x, solid))
    return out


def _params(precision, domain=(8, 8, 8)):
    from lustrine_gb300 import pbf_params
    return pbf_params(*domain, iterations=4, precision=precision)


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_batch_equals_scenes_stepped_alone(precision):
    from lustrine_gb300 import PbfSim
    scs = _scenes()
    dt = 1 / 60
    alone = []
    for sc in scs:
        sim = PbfSim(_params(precision, sc.domain), sc.n, sc.ns)
        sim.upload(sc.x, None, sc.solid if sc.ns else None)
        sim.step(dt, 5)
        assert sim.status() == 0
        alone.append(sim.download())
        sim.close()
    b = PbfSim.batch(_params(precision), [sc.domain for sc in scs], [sc.n for sc in scs],
                     [sc.ns for sc in scs])
    b.upload(np.concatenate([sc.x for sc in scs]), None,
             np.concatenate([sc.solid for sc in scs if sc.ns]))
    b.step(dt, 5)
    assert b.status() == 0
    x, v, _, _ = b.download()
    off = 0
    for sc, (xa, va, _, _) in zip(scs, alone):
        np.testing.assert_array_equal(x[off:off + sc.n], xa)
        np.testing.assert_array_equal(v[off:off + sc.n], va)
        off += sc.n
    b.close()


def test_batch_mixed_density_error_vs_fp64(orc):
    from lustrine_gb300 import PRECISION_MIXED, PbfSim
    scs = _scenes()[:4]
    b = PbfSim.batch(_params(PRECISION_MIXED), [sc.domain for sc in scs], [sc.n for sc in scs])
    b.upload(np.concatenate([sc.x for sc in scs]))
    b.step(1 / 60, 3)
    xd = b.positions_f64()
    # a lambda pass at the committed positions (dt so small that x* = x)
    p1 = _params(PRECISION_MIXED)
    p1.iterations = 1
    e = PbfSim.batch(p1, [sc.domain for sc in scs], [sc.n for sc in scs])
    x_up = xd.astype(np.float32)
    e.upload(x_up)
    e.step(1e-7)
    rho = e.density()  # the lambda pass ran at the uploaded positions
    x_eval = x_up.astype(np.float64)
    off = 0
    worst = 0.0
    for sc in scs:
        q = orc.reference_params(*sc.domain)
        q.rest_density, q.mass = p1.rest_density, p1.mass
        rho64 = orc.pbf_density(q, x_eval[off:off + sc.n])
        worst = max(worst, np.abs(rho[off:off + sc.n] - rho64).max() / np.abs(rho64).max())
        off += sc.n
    assert worst <= 1e-4, worst
    b.close()
    e.close()


def test_batch_config3_shapes_run():
    """A 64-scene slice of the 512-scene configuration steps cleanly and
    conserves mass (FP64 reduction)."""
    from lustrine_gb300 import PbfSim, pbf_params, scenes
    scs = scenes.config3(num=64)
    p = pbf_params(8, 8, 8, iterations=4)
    b = PbfSim.batch(p, [sc.domain for sc in scs], [sc.n for sc in scs])
    b.upload(np.concatenate([sc.x for sc in scs]))
    b.step(1 / 60, 3)
    assert b.status() == 0
    r = b.reduce()
    total = sum(sc.n for sc in scs) * p.mass
    assert abs(r["mass"] - total) <= 1e-12 * total
    x = b.positions()
    off = 0
    for sc in scs:
        xs = x[off:off + sc.n]
        assert (xs >= 0.5 - 1e-4).all() and (xs <= np.array(sc.domain) - 0.5 + 1e-4).all()
        off += sc.n
    b.close()


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_sharded_batches_equal_the_full_batch(precision):
    """The multi-GPU split of a batch (sharding.shard_scenes: every rank
    steps one batch of its own scenes, no collective on the data path) on one
    GPU: the batches built from shard 0 and shard 1 of 24 scenes of the
    512-scene distribution give every scene exactly what the full batch
    gives."""
    from lustrine_gb300 import PbfSim, pbf_params, scenes, sharding
    scs = scenes.config3(num=24)
    counts = [sc.n for sc in scs]
    parts = sharding.shard_scenes(counts, 2)
    assert sorted(parts[0] + parts[1]) == list(range(24)) and parts[0] and parts[1]

    def run(ids):
        sub = [scs[i] for i in ids]
        b = PbfSim.batch(pbf_params(8, 8, 8, iterations=4, precision=precision), [sc.domain for sc in sub],
                         [sc.n for sc in sub])
        b.upload(np.concatenate([sc.x for sc in sub]))
        b.step(1 / 60, 3)
        assert b.status() == 0
        x, v, _, _ = b.download()
        b.close()
        off = np.concatenate([[0], np.cumsum([sc.n for sc in sub])])
        return {i: (x[off[k]:off[k + 1]], v[off[k]:off[k + 1]]) for k, i in enumerate(ids)}

    full = run(list(range(24)))
    for ids in parts:
        for i, (x, v) in run(ids).items():
            np.testing.assert_array_equal(x, full[i][0])
            np.testing.assert_array_equal(v, full[i][1])
