"""The on-chip scene solve of batches (thread-block clusters of 16 CTAs, each
scene's lists, iterations, XSPH and commit out of distributed shared memory,
bins of scenes from a work queue).

fp32: the same bits as the per-stage batched step -- and so as every scene
stepped alone -- over several steps (direct launches, then the captured
graph): positions, velocities, lambdas, densities, neighbour lists.  The
scenes span one CTA (1 to 4,096 particles), two (4,097), several and all
sixteen (65,536) of a cluster, bins mix scenes of different sizes, and one
dense scene has lists longer than the 10 entries kept in shared memory.
Both CTA widths (512 and 1,024 threads).  Mixed precision: within the mixed
representation's contract of the FP64 oracle (density 1e-4 relative)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DT = 1.0 / 60.0


def _scenes():
    from lustrine_gb300 import scenes
    rng = np.random.default_rng(17)
    out = [scenes.batched_scene(int(n), rng) for n in (1, 2, 4095, 4096, 4097, 8192, 20000, 65536, 777, 5000)]
    # dense: spacing 0.6 at h = 1, about 18 neighbours per particle
    x = scenes.jitter(scenes.lattice((10, 10, 10), (2.0, 1.0, 2.0), spacing=0.6), 0.02, rng)
    out.append(scenes.Scene("dense", (12, 12, 12), x))
    return out


def _batch(scs, precision, onchip, iterations=4, threads=1024):
    from lustrine_gb300 import PbfSim, pbf_params
    b = PbfSim.batch(pbf_params(8, 8, 8, iterations=iterations, precision=precision), [sc.domain for sc in scs],
                     [sc.n for sc in scs])
    b.set_solver(onchip)
    assert b.solver() == ("onchip" if onchip else "stages")
    if onchip:
        b.set_onchip_threads(threads)
        lay = b.onchip_layout()
        assert lay["clusters"] >= 1 and lay["bins"] >= 1 and lay["threads"] == threads
    b.upload(np.concatenate([sc.x for sc in scs]))
    return b


@pytest.mark.parametrize("iterations,threads", [(4, 1024), (1, 512), (3, 512)])
def test_onchip_fp32_bitwise_equals_per_stage_batch(iterations, threads):
    scs = _scenes()
    a = _batch(scs, 0, False, iterations)
    b = _batch(scs, 0, True, iterations, threads)
    for step in range(4):
        a.step(DT)
        b.step(DT)
        assert a.status() == b.status()
        xa, va, la, ra = a.download(lambdas=True, density=True)
        xb, vb, lb, rb = b.download(lambdas=True, density=True)
        np.testing.assert_array_equal(xb, xa, err_msg=f"step {step}")
        np.testing.assert_array_equal(vb, va, err_msg=f"step {step}")
        np.testing.assert_array_equal(lb, la, err_msg=f"step {step}")
        np.testing.assert_array_equal(rb, ra, err_msg=f"step {step}")
    ca, ia = a.neighbors(cap=64)
    cb, ib = b.neighbors(cap=64)
    np.testing.assert_array_equal(cb, ca)
    assert ca.max() > 10  # the dense scene reads entries past the shared-memory ones
    for i in range(len(ca)):
        assert np.array_equal(ia[i, :ca[i]], ib[i, :cb[i]]), i
    a.close()
    b.close()


def test_onchip_fp32_equals_scenes_stepped_alone():
    from lustrine_gb300 import PbfSim, pbf_params
    scs = _scenes()
    b = _batch(scs, 0, True)
    b.step(DT, 3)
    x, v, _, _ = b.download()
    off = 0
    for sc in scs:
        s = PbfSim(pbf_params(*sc.domain, iterations=4), sc.n)
        s.upload(sc.x)
        s.step(DT, 3)
        xs, vs, _, _ = s.download()
        np.testing.assert_array_equal(x[off:off + sc.n], xs)
        np.testing.assert_array_equal(v[off:off + sc.n], vs)
        s.close()
        off += sc.n
    b.close()


def _oracle_params(orc, p, dom):
    q = orc.reference_params(*dom, p.particle_radius, p.kernel_radius / p.particle_radius)
    for f in ("rest_density", "mass", "relaxation_epsilon", "s_corr_dq", "s_corr_k", "s_corr_n",
              "c_xsph", "solid_contact", "iterations"):
        setattr(q, f, getattr(p, f))
    for ax in range(3):
        q.gravity[ax] = p.gravity[ax]
    return q


def test_onchip_mixed_step_vs_fp64_oracle(orc):
    """One mixed-precision on-chip step of every (non-dense) scene from its
    initial state against the FP64 oracle: densities within 1e-4 relative;
    positions within two units in the last place of an fp32 number of the
    box's size (the on-chip solve iterates on positions relative to the
    scene's box corner) plus 1e-5 of the FP64 displacement."""
    from lustrine_gb300 import PRECISION_MIXED
    scs = _scenes()[:-1]
    b = _batch(scs, PRECISION_MIXED, True)
    b.step(DT)
    assert b.status() == 0
    x, _, _, rho = b.download(density=True)
    off = 0
    for sc in scs:
        q = _oracle_params(orc, b.params, sc.domain)
        o = orc.pbf_step(q, DT, sc.x, np.zeros_like(sc.x))
        rho64 = np.asarray(o["density"])
        sl = slice(off, off + sc.n)
        assert np.max(np.abs(rho[sl] - rho64) / np.abs(rho64)) <= 1e-4, sc.n
        disp = np.linalg.norm(o["x"] - sc.x, axis=1)
        err = np.linalg.norm(x[sl] - o["x"], axis=1)
        ulp = 2.0 ** (np.ceil(np.log2(max(sc.domain))) - 24)
        assert np.all(err <= 2 * ulp + 1e-5 * disp), (sc.n, err.max(), ulp)
        off += sc.n
    b.close()


def test_onchip_profile_and_unsupported_batches():
    from lustrine_gb300 import LustrineError, PbfSim, pbf_params, scenes
    scs = _scenes()[:3]
    b = _batch(scs, 0, True)
    b.step(DT)
    prof = b.profile_step(DT)
    assert prof["solve"][1] == 1 and prof["solve"][0] > 0 and prof["delta"][1] == 0
    b.close()
    # static particles: the per-stage path only
    rng = np.random.default_rng(3)
    solid, _ = scenes.heightmap_solids(16, 600, origin=(0, 0, 0), rng=rng, max_height=3)
    x = scenes.jitter(scenes.lattice((8, 8, 8), (4, 3, 4)), 0.05, rng)
    s = PbfSim.batch(pbf_params(16, 14, 16, iterations=4), [(16, 14, 16)], [len(x)], [len(solid)])
    assert s.solver() == "stages"
    with pytest.raises(LustrineError) as e:
        s.set_solver(True)
    assert e.value.code == 6
    s.close()
