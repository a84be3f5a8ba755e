"""Hashed grid (buckets of packed cell coordinates instead of a dense cell
table) for domains whose dense table would not fit: the 4096 x 256 x 4096
box has 4.3e9 cells.

- On a small scene the hashed walk visits the same particles in the same
  order as the dense one, so the first step is bit-identical (positions,
  velocities, lambdas, densities, neighbour lists) in both precisions, and
  later steps (whose within-cell order follows the previous sort) stay within
  1e-5 of the box size.
- Far from the origin in the large box (picked hashed automatically), mixed
  precision keeps the density within 1e-4 relative of the FP64 oracle, both
  for the lambda pass at given positions and along a 3-step trajectory
  (the oracle runs in coordinates shifted by an integer corner, exact in
  float64)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _solid_scene():
    from lustrine_gb300 import scenes
    rng = np.random.default_rng(7)
    x = scenes.jitter(scenes.lattice((12, 10, 12), (6, 4, 6)), 0.05, rng)
    solid, _ = scenes.heightmap_solids(24, 1500, origin=(0, 0, 0), rng=rng, max_height=5)
    return scenes.Scene("small_solids", (24, 20, 24), x, solid, dt=1 / 60, iterations=4)


def _run(sc, precision, grid_mode, steps):
    from lustrine_gb300 import PbfSim, pbf_params
    p = pbf_params(*sc.domain, iterations=sc.iterations, precision=precision, grid_mode=grid_mode)
    sim = PbfSim(p, sc.n, sc.ns)
    sim.upload(sc.x, None, sc.solid)
    sim.step(sc.dt, steps)
    assert sim.status() == 0
    out = sim.download(lambdas=True, density=True)
    cnt, idx = sim.neighbors()
    sim.close()
    return out, cnt, idx


@pytest.mark.parametrize("precision", [0, 1])
def test_hashed_first_step_bitwise_equals_dense(precision):
    from lustrine_gb300._lib import GRID_DENSE, GRID_HASHED
    sc = _solid_scene()
    (xd, vd, ld, rd), cd, id_ = _run(sc, precision, GRID_DENSE, 1)
    (xh, vh, lh, rh), ch, ih = _run(sc, precision, GRID_HASHED, 1)
    np.testing.assert_array_equal(xh, xd)
    np.testing.assert_array_equal(vh, vd)
    np.testing.assert_array_equal(lh, ld)
    np.testing.assert_array_equal(rh, rd)
    np.testing.assert_array_equal(ch, cd)
    np.testing.assert_array_equal(ih, id_)


@pytest.mark.parametrize("precision", [0, 1])
def test_hashed_rollout_close_to_dense(precision):
    from lustrine_gb300._lib import GRID_DENSE, GRID_HASHED
    sc = _solid_scene()
    (xd, vd, _, _), _, _ = _run(sc, precision, GRID_DENSE, 8)
    (xh, vh, _, _), _, _ = _run(sc, precision, GRID_HASHED, 8)
    assert np.abs(xh - xd).max() <= 1e-5 * max(sc.domain)


def test_dense_grid_refused_for_the_large_box():
    from lustrine_gb300 import LustrineError, PbfSim, pbf_params
    from lustrine_gb300._lib import GRID_DENSE
    with pytest.raises(LustrineError):
        PbfSim(pbf_params(4096, 256, 4096, grid_mode=GRID_DENSE), 10)


BOX = (4096, 256, 4096)
CORNER = np.array([3980.0, 90.0, 3990.0])


def _far_blob():
    from lustrine_gb300 import scenes
    rng = np.random.default_rng(44)
    return scenes.jitter(scenes.lattice((20, 20, 20), tuple(CORNER + 10.0)), 0.2, rng)


def _oracle_params(orc, p, dom):
    q = orc.reference_params(*dom, p.particle_radius, p.kernel_radius / p.particle_radius)
    for f in ("rest_density", "mass", "relaxation_epsilon", "s_corr_dq", "s_corr_k", "s_corr_n",
              "c_xsph", "solid_contact", "iterations"):
        setattr(q, f, getattr(p, f))
    for a in range(3):
        q.gravity[a] = p.gravity[a]
    return q


def test_far_blob_lambda_pass_density_vs_fp64(orc):
    from lustrine_gb300 import PRECISION_MIXED, PbfSim, pbf_params
    x = _far_blob()
    p = pbf_params(*BOX, iterations=1, precision=PRECISION_MIXED)
    sim = PbfSim(p, len(x))
    sim.upload(x)
    sim.step(1e-7)
    assert sim.status() == 0
    rho = sim.density()
    sim.close()
    q = _oracle_params(orc, p, (60, 60, 60))
    rho64 = orc.pbf_density(q, x.astype(np.float64) - CORNER)
    err = np.abs(rho - rho64).max() / np.abs(rho64).max()
    assert err <= 1e-4, err


def test_far_blob_trajectory_vs_fp64(orc):
    from lustrine_gb300 import PRECISION_FP32, PRECISION_MIXED, PbfSim, pbf_params
    x0 = _far_blob()
    dt, steps = 1 / 60, 3
    q = None
    res = {}
    for prec in (PRECISION_FP32, PRECISION_MIXED):
        p = pbf_params(*BOX, iterations=4, precision=prec)
        sim = PbfSim(p, len(x0))
        sim.upload(x0)
        sim.step(dt, steps)
        assert sim.status() == 0
        res[prec] = sim.positions_f64()
        sim.close()
        q = _oracle_params(orc, p, (60, 60, 60))
    x = x0.astype(np.float64) - CORNER
    v = np.zeros_like(x)
    for _ in range(steps):
        o = orc.pbf_step(q, dt, x, v)
        x, v = o["x"], o["v"]
    rho_ref = orc.pbf_density(q, x)
    errs = {}
    for prec, xg in res.items():
        xg = xg - CORNER
        rho = orc.pbf_density(q, xg)
        errs[prec] = (np.abs(xg - x).max(), np.abs(rho - rho_ref).max() / np.abs(rho_ref).max())
    assert errs[PRECISION_MIXED][0] <= 1e-4, errs
    assert errs[PRECISION_MIXED][1] <= 1e-4, errs
    # plain fp32 rounds positions to 2.4e-4 at x ~ 4000
    assert errs[PRECISION_FP32][0] > errs[PRECISION_MIXED][0], errs
