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

Tolerances: per particle, positions within 1e-5 of max(h, its FP64
displacement) plus half a unit in the last place of an fp32 number of the
coordinate's size per rounding of the stored position (fp32 rounds it at the
prediction, at every Jacobi update and at the commit; mixed precision keeps
cell-relative offsets and rounds the absolute position once, at the download,
counted twice); velocities the same over dt; densities within 1e-5 relative in fp32 and 1e-4 in mixed precision
(its contract, also 3,900+ cells from the origin), lambdas within that
density tolerance carried through lambda = -(rho / rho0 - 1) / (S + eps) plus
1e-4 of max |lambda| (near the rest density lambda is a small difference);
neighbour sets equal to the FP64 sets of the predicted positions except for
pairs whose FP64 distance is within 1e-5 h of h (enumerated, and bounded)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def position_bound(x64, x0, roundings, h=1.0):
    """Per-particle bound on |x - x64|: 1e-5 of max(h, the FP64 displacement)
    plus half an fp32 unit in the last place of the coordinates' size per
    rounding of the stored position (normwise over the three axes)."""
    disp = np.linalg.norm(np.asarray(x64, np.float64) - np.asarray(x0, np.float64), axis=1)
    ulp = np.spacing(np.abs(np.asarray(x64, np.float32)).max(axis=1)).astype(np.float64)
    return 1e-5 * np.maximum(h, disp) + np.sqrt(3.0) * 0.5 * roundings * ulp


def roundings_of(precision, iterations):
    return 2 if precision else iterations + 2


def check_positions(x, x64, x0, v, v64, dt, roundings, h=1.0):
    bound = position_bound(x64, x0, roundings, h)
    err = np.linalg.norm(np.asarray(x, np.float64) - x64, axis=1)
    assert np.all(err <= bound), (err.max(), int(np.argmax(err / bound)))
    verr = np.linalg.norm(np.asarray(v, np.float64) - v64, axis=1)
    assert np.all(verr <= bound / dt), (verr.max(), int(np.argmax(verr / bound)))


def check_sets(cnt, idx, xs64, h, solid=None):
    """Every GPU list holds each pair the FP64 predicted positions put
    closer than h (1 - 1e-5), and nothing farther than h (1 + 1e-5): pairs in
    between are decided by fp32 rounding.  Returns how many pairs fall there
    (fluid pairs counted from both sides).  Ids: fluid 0..n-1, solids n + k."""
    from scipy.spatial import cKDTree
    n = len(xs64)
    pts = xs64 if solid is None or len(solid) == 0 else np.concatenate([xs64, np.asarray(solid, np.float64)])
    N = len(pts)
    pr = cKDTree(pts).query_pairs(r=h * (1 + 1e-5), output_type="ndarray").astype(np.int64)
    pr = pr[pr[:, 0] < n]  # at least one fluid particle (query_pairs gives i < j)
    r = np.linalg.norm(pts[pr[:, 0]] - pts[pr[:, 1]], axis=1)
    both = pr[:, 1] < n
    # directed pairs: i -> j always, j -> i when j is fluid
    src = np.concatenate([pr[:, 0], pr[both, 1]])
    dst = np.concatenate([pr[:, 1], pr[both, 0]])
    rr = np.concatenate([r, r[both]])
    band = np.abs(rr - h) <= 1e-5 * h
    sure = np.sort(src[~band] * N + dst[~band])
    allowed = np.sort(src * N + dst)
    rows = np.repeat(np.arange(n, dtype=np.int64), cnt)
    cols = idx[np.arange(idx.shape[1])[None, :] < cnt[:, None]].astype(np.int64)
    keep = cols != rows  # PBF lists report the particle itself first
    got = np.sort(rows[keep] * N + cols[keep])
    assert len(got) == len(np.unique(got))
    assert np.all(np.isin(sure, got)), int((~np.isin(sure, got)).sum())
    assert np.all(np.isin(got, allowed)), int((~np.isin(got, allowed)).sum())
    return int(band.sum())


def predicted64(x0, v0, p, dt, domain):
    """FP64 prediction: v += g dt, x* = clamp(x + v dt, r, L - r) per axis."""
    v = np.asarray(v0, np.float64) + np.array([p.gravity[0], p.gravity[1], p.gravity[2]], np.float64) * dt
    xs = np.asarray(x0, np.float64) + v * dt
    lo, hi = p.particle_radius, np.array(domain, np.float64) - p.particle_radius
    return np.clip(xs, lo, hi)


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
        cnt, idx = sim.neighbors(cap=16)  # counts in full, entries up to 16 (7 at most here)
        r = sim.reduce()
    assert cnt.max() <= 16
    q = _oracle_params(orc, p, sc.domain)
    o = orc.pbf_step(q, sc.dt, sc.x, np.zeros_like(sc.x), solid=sc.solid if sc.ns else None)
    check_positions(x, o["x"], sc.x, v, o["v"], sc.dt, roundings_of(precision, sc.iterations))
    xs64 = predicted64(sc.x, np.zeros_like(sc.x), p, sc.dt, sc.domain)
    edge = check_sets(cnt, idx, xs64, p.kernel_radius, sc.solid if sc.ns else None)
    # the lattice puts six neighbours of every particle at r = h +- 0.07 (jitter
    # +-0.05 per axis): about 1.2e-3 pairs per particle fall within 1e-5 h of h
    assert edge <= 3e-3 * sc.n, edge
    tol = 1e-4 if precision else 1e-5  # the mixed representation's density contract: 1e-4
    rmax = np.abs(o["density"]).max()
    assert np.abs(rho - o["density"]).max() <= tol * rmax
    # lambda = -(rho / rho0 - 1) / (S + eps): the density tolerance carried through
    lam_tol = tol * rmax / (q.rest_density * q.relaxation_epsilon) + 1e-4 * np.abs(o["lambdas"]).max()
    assert np.abs(lam - o["lambdas"]).max() <= lam_tol
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


@pytest.mark.parametrize("mixed", [0, 1, 2])
def test_config3_full_batch_step_vs_fp64_oracle(orc, mixed):
    """All 512 scenes of config 3 in one batched step (fp32, mixed with
    cell-relative iterations, mixed with scene-frame iterations): status, FP64
    mass, every scene inside its box, and its smallest, median and largest
    scenes against the oracle stepping each alone (densities within 1e-5
    relative in fp32, 1e-4 in the mixed representations)."""
    from lustrine_gb300 import PbfSim, pbf_params, scenes
    scs = scenes.config3()
    assert len(scs) == 512
    p = pbf_params(8, 8, 8, iterations=4, precision=mixed)
    with PbfSim.batch(p, [sc.domain for sc in scs], [sc.n for sc in scs]) as b:
        b.upload(np.concatenate([sc.x for sc in scs]))
        b.step(scs[0].dt)
        assert b.status() == 0
        x, v, _, rho = b.download(density=True)
        r = b.reduce()
    total = sum(sc.n for sc in scs)
    assert abs(r["mass"] - total * p.mass) <= 1e-9 * total * p.mass
    off = np.concatenate([[0], np.cumsum([sc.n for sc in scs])])
    for k, sc in enumerate(scs):
        xs = x[off[k]:off[k + 1]]
        assert (xs >= 0.5 - 1e-4).all() and (xs <= np.array(sc.domain) - 0.5 + 1e-4).all(), k
    order = np.argsort([sc.n for sc in scs])
    for k in (order[0], order[len(order) // 2], order[-1]):
        sc = scs[k]
        q = _oracle_params(orc, p, sc.domain)
        o = orc.pbf_step(q, sc.dt, sc.x, np.zeros_like(sc.x))
        # the scene frame rounds the stored position like fp32 does
        check_positions(x[off[k]:off[k + 1]], o["x"], sc.x, v[off[k]:off[k + 1]], o["v"], sc.dt,
                        roundings_of(mixed == 1, 4))
        tol = 1e-4 if mixed else 1e-5
        rho64 = np.asarray(o["density"])
        assert np.max(np.abs(rho[off[k]:off[k + 1]] - rho64) / np.abs(rho64)) <= tol, k


def test_config1_reference_semantics_full_step_vs_oracle(orc):
    """Config 1 (262,144 fluid + 50,000 static particles) under the
    reference's own step (mode R: its cubic kernel, double self density,
    lambda by list position, 0.01 floor snap, one pass) against the oracle's
    restatement of that step, pinned to the compiled reference: neighbour
    counts equal, lambdas, positions and velocities within 1e-5 relative
    (per particle, normwise), and bitwise equal for all but a few particles
    (the reference's powf misrounds ~0.07 % of the s_corr powers, which the
    GPU evaluates exactly)."""
    from conftest import phys_params
    from lustrine_gb300 import PbfSim, reference_params, scenes
    sc = scenes.config1()
    p = phys_params(reference_params(*sc.domain))
    p.max_neighbors = 64
    with PbfSim(p, sc.n, sc.ns) as sim:
        sim.upload(sc.x, None, sc.solid)
        sim.step(sc.dt)
        assert sim.status() == 0
        x, v, lam, _ = sim.download(lambdas=True)
        cnt, idx = sim.neighbors(cap=64)
    q = phys_params(orc.reference_params(*sc.domain))
    q.jacobi = 1
    o = orc.compat_step(q, sc.dt, sc.x, np.zeros_like(sc.x), solid=sc.solid, cap=64)
    assert np.array_equal(cnt, o["nbr_count"])
    # the full lists, in the reference's order (cell order, then ascending id)
    ref_idx = o["nbr_idx"]
    for i in range(sc.n):
        assert np.array_equal(idx[i, :cnt[i]], ref_idx[i, :cnt[i]]), i

    def rel(a, b):
        a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
        nb = np.linalg.norm(b.reshape(len(b), -1), axis=1)
        floor = 1e-3 * np.sqrt(np.mean(nb ** 2))
        return np.linalg.norm((a - b).reshape(len(b), -1), axis=1) / np.maximum(nb, floor)

    assert rel(x, o["x"]).max() <= 1e-5
    assert rel(v, o["v"]).max() <= 1e-5
    lo = o["lambdas"][:sc.n]
    assert np.all(np.abs(lam - lo) <= 1e-5 * np.maximum(np.abs(lo), 1e-3 * np.abs(lo).max()))
    same = np.mean(np.all(x == o["x"], axis=1) & np.all(v == o["v"], axis=1))
    assert same >= 0.99, same
