"""The benchmark configurations at full size, one step each, against the FP64
oracle, plus the size-independent properties (status, particles inside the
box, FP64 mass):

* config 1: 262,144 fluid + 50,000 static particles, fp32 and mixed precision;
* config 2: 2,097,152 particles, 6 iterations;
* config 4: 4,194,304 particles in 16 blobs on the hashed grid, mixed
  precision; the blobs lie at least 2 cells apart, so a blob's step does not
  depend on the others: the one farthest from the origin is checked against
  the oracle stepping that blob alone, in a box shifted by whole cells in x
  and z to its neighbourhood (y and the floor kept).

Tolerances as the small-scene step tests: positions within 2e-5 of the box
size (per second for velocities), densities within 1e-5 relative in fp32
and 1e-4 in mixed precision (its contract, also 3,900+ cells from the
origin), lambdas within that density tolerance carried through
lambda = -(rho / rho0 - 1) / (S + eps) plus 1e-4 of max |lambda| (near the rest
density lambda is a small difference), neighbour counts equal except for
pairs at r = h within rounding."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _oracle_params(orc, p, dom):
    q = orc.reference_params(*dom, p.particle_radius, p.kernel_radius / p.particle_radius)
    for f in ("rest_density", "mass", "relaxation_epsilon", "s_corr_dq", "s_corr_k", "s_corr_n",
              "c_xsph", "solid_contact", "iterations"):
        setattr(q, f, getattr(p, f))
    for a in range(3):
        q.gravity[a] = p.gravity[a]
    return q


def _step_and_check(orc, sc, precision):
    from lustrine_gb300 import PbfSim, pbf_params
    p = pbf_params(*sc.domain, iterations=sc.iterations, c_xsph=sc.c_xsph, precision=precision)
    with PbfSim(p, sc.n, sc.ns) as sim:
        sim.upload(sc.x, None, sc.solid if sc.ns else None)
        sim.step(sc.dt)
        assert sim.status() == 0
        x, v, lam, rho = sim.download(lambdas=True, density=True)
        cnt, _ = sim.neighbors(cap=16)  # counts in full, entries up to 16 (7 at most here)
        r = sim.reduce()
    q = _oracle_params(orc, p, sc.domain)
    o = orc.pbf_step(q, sc.dt, sc.x, np.zeros_like(sc.x), solid=sc.solid if sc.ns else None)
    L = max(sc.domain)
    assert np.abs(x - o["x"]).max() <= 2e-5 * L
    assert np.abs(v - o["v"]).max() <= 2e-5 * L / sc.dt
    tol = 1e-4 if precision else 1e-5  # the mixed representation's density contract: 1e-4
    rmax = np.abs(o["density"]).max()
    assert np.abs(rho - o["density"]).max() <= tol * rmax
    # lambda = -(rho / rho0 - 1) / (S + eps): the density tolerance carried through
    lam_tol = tol * rmax / (q.rest_density * q.relaxation_epsilon) + 1e-4 * np.abs(o["lambdas"]).max()
    assert np.abs(lam - o["lambdas"]).max() <= lam_tol
    assert np.mean(cnt == o["nbr_count"]) > 0.999
    lo, hi = p.particle_radius, np.array(sc.domain, np.float32) - p.particle_radius
    assert (x >= lo - 1e-4).all() and (x <= hi + 1e-4).all()
    assert abs(r["mass"] - sc.n * p.mass) <= 1e-9 * sc.n * p.mass


@pytest.mark.parametrize("mixed", [False, True])
def test_config1_full_step_vs_fp64_oracle(orc, mixed):
    from lustrine_gb300 import PRECISION_FP32, PRECISION_MIXED, scenes
    _step_and_check(orc, scenes.config1(), PRECISION_MIXED if mixed else PRECISION_FP32)


def test_config2_full_step_vs_fp64_oracle(orc):
    from lustrine_gb300 import PRECISION_FP32, scenes
    _step_and_check(orc, scenes.config2(), PRECISION_FP32)


def test_config4_full_mixed_step_blob_vs_fp64_oracle(orc):
    from lustrine_gb300 import PRECISION_MIXED, PbfSim, pbf_params, scenes
    sc = scenes.config4()
    blob = 64 ** 3
    assert sc.n == 16 * blob
    p = pbf_params(*sc.domain, iterations=sc.iterations, c_xsph=sc.c_xsph, precision=PRECISION_MIXED)
    with PbfSim(p, sc.n) as sim:
        sim.upload(sc.x)
        sim.step(sc.dt)
        assert sim.status() == 0
        xg = sim.positions_f64()
        r = sim.reduce()
    assert abs(r["mass"] - sc.n * p.mass) <= 1e-9 * sc.n * p.mass
    assert (xg >= 0.5 - 1e-4).all() and (xg <= np.array(sc.domain) - 0.5 + 1e-4).all()
    # the blob farthest from the origin (x, z), away from the side walls
    lows = sc.x.reshape(16, blob, 3).min(1)
    far = [b for b in range(16) if lows[b, 0] >= 8 and lows[b, 2] >= 8
           and lows[b, 0] + 72 <= sc.domain[0] and lows[b, 2] + 72 <= sc.domain[2]]
    b = max(far, key=lambda k: lows[k, 0] + lows[k, 2])
    assert lows[b, 0] + lows[b, 2] > 3900
    shift = np.array([np.floor(lows[b, 0]) - 8, 0.0, np.floor(lows[b, 2]) - 8])
    dom = (80, sc.domain[1], 80)
    q = _oracle_params(orc, p, dom)
    x0 = sc.x[b * blob:(b + 1) * blob].astype(np.float64) - shift
    o = orc.pbf_step(q, sc.dt, x0, np.zeros_like(x0))
    mine = xg[b * blob:(b + 1) * blob] - shift
    assert np.abs(mine - o["x"]).max() <= 1e-4
    rho_ref = orc.pbf_density(q, o["x"])
    rho = orc.pbf_density(q, mine)
    assert np.abs(rho - rho_ref).max() <= 1e-4 * np.abs(rho_ref).max()
