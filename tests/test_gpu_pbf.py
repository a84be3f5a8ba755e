"""GPU PBF step against the CPU oracle (the FP64 restatement of the same
step).  Tolerances: one step -- positions within 2e-5 of the box size,
lambdas within 1e-4 of max |lambda|, densities within 1e-5 relative; the
mixed-precision representation keeps the density within 1e-4 relative of the
FP64 oracle evaluated at the GPU's own positions."""
import numpy as np
import pytest

from conftest import rows_sets

pytestmark = pytest.mark.gpu


def _params(sc, **kw):
    from lustrine_gb300 import pbf_params
    p = pbf_params(*sc.domain, iterations=sc.iterations, c_xsph=sc.c_xsph)
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def _oracle_params(orc, p):
    q = orc.reference_params(p.domain[0], p.domain[1], p.domain[2], p.particle_radius,
                             p.kernel_radius / p.particle_radius)
    for f in ("rest_density", "mass", "relaxation_epsilon", "s_corr_dq", "s_corr_k", "s_corr_n",
              "c_xsph", "solid_contact", "iterations"):
        setattr(q, f, getattr(p, f))
    for a in range(3):
        q.gravity[a] = p.gravity[a]
    return q


def _small_solid_scene():
    from lustrine_gb300 import scenes
    rng = np.random.default_rng(5)
    x = scenes.jitter(scenes.lattice((12, 10, 12), (6, 4, 6)), 0.05, rng)
    solid, _ = scenes.heightmap_solids(24, 1500, origin=(0, 0, 0), rng=rng, max_height=5)
    return scenes.Scene("small_solids", (24, 20, 24), x, solid, dt=1 / 60, iterations=4)


@pytest.mark.parametrize("which", ["c0", "solids"])
def test_pbf_one_step_matches_fp64_oracle(orc, which):
    from lustrine_gb300 import PbfSim, scenes
    sc = scenes.config0(seed=21) if which == "c0" else _small_solid_scene()
    p = _params(sc)
    sim = PbfSim(p, sc.n, sc.ns)
    sim.upload(sc.x, None, sc.solid if sc.ns else None)
    sim.step(sc.dt)
    assert sim.status() == 0
    x, v, lam, rho = sim.download(lambdas=True, density=True)
    q = _oracle_params(orc, p)
    o = orc.pbf_step(q, sc.dt, sc.x, np.zeros_like(sc.x), solid=sc.solid if sc.ns else None)
    L = max(sc.domain)
    assert np.abs(x - o["x"]).max() <= 2e-5 * L
    assert np.abs(v - o["v"]).max() <= 2e-5 * L / sc.dt
    assert np.abs(lam - o["lambdas"]).max() <= 1e-4 * np.abs(o["lambdas"]).max()
    assert np.abs(rho - o["density"]).max() <= 1e-5 * np.abs(o["density"]).max()
    cnt, _ = sim.neighbors()
    # neighbour counts agree except for pairs at r = h within rounding
    assert np.mean(cnt == o["nbr_count"]) > 0.999
    sim.close()


def test_pbf_neighbour_sets_exact_at_same_positions(orc):
    """With iterations = 1, no gravity and dt tiny, x* = x: the neighbour sets
    of the PBF lists equal the oracle's set of particles within h."""
    from lustrine_gb300 import PbfSim, scenes
    sc = _small_solid_scene()
    p = _params(sc, iterations=1)
    p.gravity[1] = 0.0
    sim = PbfSim(p, sc.n, sc.ns)
    sim.upload(sc.x, None, sc.solid)
    sim.step(1e-6)
    cnt, idx = sim.neighbors()
    q = orc.reference_params(*sc.domain)
    ocnt, oidx = orc.compat_neighbors(q, sc.x, sc.solid)
    for a, b in zip(rows_sets(cnt, idx), rows_sets(ocnt, oidx)):
        assert np.array_equal(a, b)
    sim.close()


def _density_at(sim_params, x, n):
    """GPU density of the lambda pass at positions x: one step with dt so
    small that x* = x in float (v dt ~ 1e-14), iterations = 1."""
    from lustrine_gb300 import PbfSim
    sim = PbfSim(sim_params, n)
    sim.upload(x)
    sim.step(1e-7)
    rho = sim.density()
    st = sim.status()
    sim.close()
    return rho, st


@pytest.mark.parametrize("offset", [0.0, 3900.0])
def test_density_error_vs_fp64_near_and_far_from_origin(orc, offset):
    """The same 10k block at the origin and 3,900 cells away: the lambda pass
    at given positions stays within 1e-4 relative density error of FP64 in
    both precisions (pair offsets of nearby fp32 positions are exact; the
    resolution plain fp32 loses far away shows along a trajectory, which
    tests/test_gpu_hashed.py::test_far_blob_trajectory_vs_fp64 checks)."""
    from lustrine_gb300 import PRECISION_MIXED, pbf_params, scenes
    rng = np.random.default_rng(31)
    # the block starts one cell above the floor so no particle is clamped by
    # the prediction (the oracle's density is evaluated at the given positions)
    x = scenes.jitter(scenes.lattice((20, 25, 20), (10 + offset, 1, 10)), 0.2, rng)
    dom = (int(offset) + 40, 40, 40)
    errs = {}
    for prec in (0, PRECISION_MIXED):
        p = pbf_params(*dom, iterations=1, precision=prec)
        rho, st = _density_at(p, x, len(x))
        assert st == 0
        q = _oracle_params(orc, p)
        rho64 = orc.pbf_density(q, x.astype(np.float64))
        errs[prec] = np.abs(rho - rho64).max() / np.abs(rho64).max()
    assert errs[PRECISION_MIXED] <= 1e-4, errs
    assert errs[0] <= 1e-4, errs


def test_mixed_one_step_matches_fp64_oracle(orc):
    from lustrine_gb300 import PRECISION_MIXED, PbfSim, scenes
    sc = scenes.config0(seed=23)
    p = _params(sc, precision=PRECISION_MIXED)
    sim = PbfSim(p, sc.n)
    sim.upload(sc.x)
    sim.step(sc.dt)
    x, v, lam, rho = sim.download(lambdas=True, density=True)
    o = orc.pbf_step(_oracle_params(orc, p), sc.dt, sc.x, np.zeros_like(sc.x))
    err = np.abs(x - o["x"])
    i = int(np.argmax(err.max(1)))
    assert err.max() <= 2e-5 * 40, (err.max(), i, x[i], o["x"][i], sc.x[i])
    assert np.abs(v - o["v"]).max() <= 2e-5 * 40 / sc.dt
    assert np.abs(rho - o["density"]).max() <= 1e-5 * np.abs(o["density"]).max()
    sim.close()


def test_mixed_and_plain_agree_near_origin(orc):
    from lustrine_gb300 import PRECISION_MIXED, PbfSim, scenes
    sc = scenes.config0(seed=23)
    out = []
    for prec in (0, PRECISION_MIXED):
        sim = PbfSim(_params(sc, precision=prec), sc.n)
        sim.upload(sc.x)
        sim.step(sc.dt, 2)
        out.append(sim.positions())
        sim.close()
    err = np.abs(out[0] - out[1])
    i = int(np.argmax(err.max(1)))
    assert err.max() < 1e-3, (err.max(), i, out[0][i], out[1][i], sc.x[i])


def test_autotune_keeps_state_and_all_shapes_agree():
    from lustrine_gb300 import PbfSim, scenes
    sc = scenes.config0(seed=27)
    sim = PbfSim(_params(sc), sc.n)
    sim.upload(sc.x)
    sim.step(sc.dt, 2)
    before = sim.download()
    best, ms = sim.autotune(sc.dt, steps=2)
    after = sim.download()
    assert np.array_equal(before[0], after[0]) and np.array_equal(before[1], after[1])
    assert best["block"] in (64, 128, 256) and best["unroll"] in (1, 2, 4, 8) and ms > 0
    assert sim.get_tuning() == best
    # every launch shape computes the same step (same summation order)
    ref = None
    for blk, unr in ((64, 1), (128, 2), (256, 4), (128, 8)):
        sim.upload(before[0], before[1])
        sim.set_tuning(blk, unr, blk)
        sim.step(sc.dt)
        x = sim.positions()
        if ref is None:
            ref = x
        assert np.abs(x - ref).max() <= 1e-5
    sim.close()


@pytest.mark.parametrize("with_solids", [False, True])
def test_two_particles_per_thread_give_the_same_bits(with_solids):
    """The lambda and delta-p passes with two particles per thread (their
    lists walked together, the shorter one padded with the sentinel, whose
    terms are exact zeros) compute the same fp32 bits as one per thread."""
    from lustrine_gb300 import PbfSim, scenes
    rng = np.random.default_rng(8)
    if with_solids:
        solid, _ = scenes.heightmap_solids(16, 600, origin=(0, 0, 0), rng=rng, max_height=3)
        x = scenes.jitter(scenes.lattice((8, 8, 8), (4, 3, 4)), 0.05, rng)
        sc = scenes.Scene("solids", (16, 14, 16), x, solid)
    else:
        sc = scenes.config0(seed=31)
    res = []
    for unroll, ppt in ((1, 1), (2, 1), (1, 2), (2, 2)):
        sim = PbfSim(_params(sc), sc.n, sc.ns)
        sim.upload(sc.x, None, sc.solid if sc.ns else None)
        sim.set_tuning(128, unroll, 128, 2, ppt)
        assert sim.get_tuning()["particles_per_thread"] == ppt
        sim.step(sc.dt, 4)
        assert sim.status() == 0
        res.append(sim.download(lambdas=True, density=True))
        sim.close()
    for r in res[1:]:
        for a, b in zip(res[0], r):
            np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("precision", [1, 2])
def test_gathers_in_flight_give_the_same_bits_with_compensated_sums(precision):
    """The mixed representations sum densities with Kahan compensation; a walk
    with more gathers in flight visits more sentinel entries (exact zero
    terms), which leave the compensated sum untouched, so 1, 2, 4 and 8
    gathers in flight give the same bits (column lists)."""
    from lustrine_gb300 import LISTS_COLUMN, PbfSim, scenes
    sc = scenes.config0(seed=33)
    res = []
    for unroll in (1, 2, 4, 8):
        sim = PbfSim(_params(sc, precision=precision), sc.n)
        sim.upload(sc.x)
        sim.set_tuning(128, unroll, 128, unroll, 1, list_format=LISTS_COLUMN)
        sim.step(sc.dt, 4)
        assert sim.status() == 0
        res.append(sim.download(lambdas=True, density=True))
        sim.close()
    for r in res[1:]:
        for a, b in zip(res[0], r):
            np.testing.assert_array_equal(a, b)


def test_graph_and_direct_launches_are_identical():
    from lustrine_gb300 import PbfSim, scenes
    sc = scenes.config0(seed=24)
    res = []
    for g in (True, False):
        sim = PbfSim(_params(sc, use_graph=1 if g else 0), sc.n)
        sim.upload(sc.x)
        sim.step(sc.dt, 5)
        res.append(sim.download())
        sim.close()
    assert np.array_equal(res[0][0], res[1][0]) and np.array_equal(res[0][1], res[1][1])


def test_rollout_statistics_vs_fp64_oracle(orc):
    """Config 0's 100 steps of the 10k dam break (collapse and splash) on the
    GPU against the FP64 oracle.  (1) Every step from the GPU's own state: the
    GPU's next positions and velocities against one FP64 step from the same
    state, within 2e-5 of the box size (per second for velocities) -- the
    chaos-free check.  (2) The free trajectories every 20 steps: kinetic
    energy, centre of mass and max density error within twice the largest
    deviation of three FP64 runs started from positions perturbed by 1e-6,
    1e-5 and 1e-4 relative, or within a floor of 2 % (energy), 0.02 (centre of
    mass, box of 40) and 3 % (density error): the flow is chaotic and the max
    density error an extreme over 10,000 particles."""
    from lustrine_gb300 import PbfSim, scenes
    sc = scenes.config0(seed=25)
    p = _params(sc, max_neighbors=128)
    q = _oracle_params(orc, p)
    L = max(sc.domain)
    sim = PbfSim(p, sc.n)
    sim.upload(sc.x)
    rng = np.random.default_rng(7)
    x0 = sc.x.astype(np.float64)
    pert = rng.uniform(-1.0, 1.0, x0.shape)
    runs = [(x0 * (1.0 + e * pert), np.zeros_like(x0)) for e in (0.0, 1e-6, 1e-5, 1e-4)]
    xg, vg = sc.x, np.zeros_like(sc.x)

    def stats(x, v, rho):
        return np.array([0.5 * q.mass * (v ** 2).sum(), *x.mean(0), np.abs(rho / q.rest_density - 1).max()])

    for s in range(100):
        one = orc.pbf_step(q, sc.dt, xg, vg)
        sim.step(sc.dt)
        xg, vg, _, _ = sim.download()
        assert np.abs(xg - one["x"]).max() <= 2e-5 * L, s
        assert np.abs(vg - one["v"]).max() <= 2e-5 * L / sc.dt, s
        outs = [orc.pbf_step(q, sc.dt, x, v) for x, v in runs]
        runs = [(o["x"], o["v"]) for o in outs]
        if s % 20 == 19:
            r = sim.reduce()
            assert sim.status() == 0, s
            assert abs(r["mass"] - sc.n * q.mass) < 1e-6
            st = [stats(o["x"], o["v"], o["density"]) for o in outs]
            a, spread = st[0], np.max([np.abs(b - st[0]) for b in st[1:]], axis=0)
            g = np.array([r["kinetic"], *r["com"], r["max_density_error"]])
            band = np.maximum(2 * spread, [0.02 * a[0], 0.02, 0.02, 0.02, 0.03 * a[4]])
            assert (np.abs(g - a) <= band).all(), (s, g, a, band)
    assert (xg >= 0.5 - 1e-5).all() and (xg <= 39.5 + 1e-5).all()
    sim.close()


def test_neighbour_overflow_is_reported_not_faulted():
    from lustrine_gb300 import PbfSim, scenes
    sc = scenes.config0(seed=26)
    sim = PbfSim(_params(sc, max_neighbors=2), sc.n)
    sim.upload(sc.x)
    sim.step(sc.dt)
    assert sim.status() == 4  # LUSTRINE_ERR_NBR_OVERFLOW
    assert sim.status() == 0  # cleared
    sim.close()


def test_edge_cases_empty_single_and_no_solids():
    from lustrine_gb300 import LustrineError, PbfSim, pbf_params
    p = pbf_params(8, 8, 8)
    sim = PbfSim(p, 0, 0)
    sim.upload(np.zeros((0, 3), np.float32))
    sim.step(1 / 60)
    assert sim.positions().shape == (0, 3)
    sim.close()
    sim = PbfSim(p, 1, 0)
    sim.upload(np.array([[4.0, 4.0, 4.0]], np.float32))
    sim.step(1 / 60, 10)
    x = sim.positions()
    assert x[0, 1] < 4.0 and np.isfinite(x).all()
    sim.close()
    with pytest.raises(LustrineError):
        PbfSim(p, -1, 0)
    bad = pbf_params(8, 8, 8)
    bad.iterations = 0
    with pytest.raises(LustrineError):
        PbfSim(bad, 10, 0)


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_state_transfers_page_locked_and_pageable_agree(precision):
    """upload/download_state_async read and write page-locked host buffers
    directly from the kernels and stage pageable ones through copies: both
    give the same states."""
    torch = pytest.importorskip("torch")
    from lustrine_gb300 import PbfSim, scenes
    sc = scenes.config0(seed=29)
    p = _params(sc, precision=precision)
    a, b = PbfSim(p, sc.n), PbfSim(p, sc.n)
    for s in (a, b):
        s.upload(sc.x)
        s.step(sc.dt, 2)
    x_ref, v_ref, _, _ = a.download()
    px = torch.empty((sc.n, 3), dtype=torch.float32).pin_memory()
    pv = torch.empty((sc.n, 3), dtype=torch.float32).pin_memory()
    a.download_state_async(px.data_ptr(), pv.data_ptr())
    a.synchronize()
    np.testing.assert_array_equal(px.numpy(), x_ref)
    np.testing.assert_array_equal(pv.numpy(), v_ref)
    hx, hv = np.empty_like(x_ref), np.empty_like(v_ref)
    b.download_state_async(hx.ctypes.data, hv.ctypes.data)
    b.synchronize()
    np.testing.assert_array_equal(hx, x_ref)
    # a new state in: page-locked into a, pageable into b
    rng = np.random.default_rng(3)
    nx = (x_ref + rng.uniform(-0.05, 0.05, x_ref.shape)).astype(np.float32)
    nv = rng.normal(size=v_ref.shape).astype(np.float32)
    px.numpy()[:] = nx
    pv.numpy()[:] = nv
    a.upload_state_async(px.data_ptr(), pv.data_ptr())
    b.upload_state_async(nx.ctypes.data, nv.ctypes.data)
    for s in (a, b):
        s.step(sc.dt)
    xa, va, _, _ = a.download()
    xb, vb, _, _ = b.download()
    np.testing.assert_array_equal(xa, xb)
    np.testing.assert_array_equal(va, vb)
    # one-call frames: the state stays in the host arrays
    hx, hv = xb.copy(), vb.copy()
    px.numpy()[:] = xa
    pv.numpy()[:] = va
    for _ in range(3):
        a.step_host(sc.dt, px.data_ptr(), pv.data_ptr())
        b.step_host(sc.dt, hx.ctypes.data, hv.ctypes.data)
    np.testing.assert_array_equal(px.numpy(), hx)
    np.testing.assert_array_equal(pv.numpy(), hv)
    # device-resident steps after host frames: the page-locked download reads
    # the slots the last sort recorded, the pageable one unpermutes by id
    for s in (a, b):
        s.step(sc.dt, 2)
    a.download_state_async(px.data_ptr(), pv.data_ptr())
    a.synchronize()
    xb, vb, _, _ = b.download()
    np.testing.assert_array_equal(px.numpy(), xb)
    np.testing.assert_array_equal(pv.numpy(), vb)
    assert a.status() == 0 and b.status() == 0
    a.close()
    b.close()


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_next_step_prediction_in_commit_kernel_is_exact(precision):
    """The commit kernel predicts the next step when nothing changes in
    between; a context made to predict every step itself (re-setting its
    launch shape drops the prediction) gives the same states bit for bit,
    also across a change of dt and with static particles."""
    from lustrine_gb300 import PbfSim
    sc = _small_solid_scene()
    p = _params(sc, precision=precision)
    a, b = PbfSim(p, sc.n, sc.ns), PbfSim(p, sc.n, sc.ns)
    for s in (a, b):
        s.upload(sc.x, None, sc.solid)
    iters = p.iterations
    for k in range(7):
        dt = sc.dt if k < 4 else 0.5 * sc.dt
        a.step(dt)
        # the prediction kernel runs after an upload and a change of dt only;
        # scan 1 (tile totals counted by the prediction), sort 2, passes, commit
        assert a.launches_per_step() == 1 + 2 + 2 * iters + 1 + (k in (0, 4))
        b.set_tuning(**b.get_tuning())
        b.step(dt)
        assert b.launches_per_step() == 1 + 2 + 2 * iters + 2
    xa, va, la, ra = a.download(lambdas=True, density=True)
    xb, vb, lb, rb = b.download(lambdas=True, density=True)
    np.testing.assert_array_equal(xa, xb)
    np.testing.assert_array_equal(va, vb)
    np.testing.assert_array_equal(la, lb)
    np.testing.assert_array_equal(ra, rb)
    assert a.status() == 0 and b.status() == 0
    a.close()
    b.close()


def test_neighbour_sets_exact_on_a_grid_past_the_single_pass_scan(orc):
    """A 300 x 200 x 300 box has 18.3 M cells, past the 4,096 tiles (16.7 M
    cells) whose totals one scan block sums on its own: the tile totals are
    scanned first.  The lists still equal the oracle's sets."""
    from lustrine_gb300 import PbfSim, scenes
    rng = np.random.default_rng(12)
    x = scenes.jitter(scenes.lattice((16, 12, 16), (140, 90, 140)), 0.05, rng)
    from lustrine_gb300 import pbf_params
    p = pbf_params(300, 200, 300, iterations=1)
    p.gravity[1] = 0.0
    sim = PbfSim(p, len(x))
    sim.upload(x)
    sim.step(1e-6)
    assert sim.status() == 0
    cnt, idx = sim.neighbors()
    q = orc.reference_params(300, 200, 300)
    ocnt, oidx = orc.compat_neighbors(q, x)
    for a, b in zip(rows_sets(cnt, idx), rows_sets(ocnt, oidx)):
        assert np.array_equal(a, b)
    assert sim.query_cell_count((0, 0, 0), (300, 200, 300)) == len(x)
    sim.close()
