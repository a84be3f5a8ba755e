"""The CPU oracle against the reference's golden vectors (no GPU).

The fixtures were written by running the reference's own code
(tests/golden/make_golden.py); these tests pin the C restatement to them
bit for bit, so it can serve as the checker of the CUDA kernels.
"""
import numpy as np
import pytest

from conftest import csr_sets, golden, phys_params, rows_sets


def test_counting_sort_matches_reference_unit_test(orc):
    # experiments/unit_tests/main.cpp:46-89: the permutation sorts the keys
    g = golden("counting_sort.npz")
    perm = orc.counting_sort(g["keys"], int(g["num_cells"]))
    assert np.array_equal(perm, g["perm"])
    assert np.array_equal(g["keys"][perm], np.sort(g["keys"], kind="stable"))
    # stability: equal keys keep input order
    k = g["keys"][perm]
    same = k[1:] == k[:-1]
    assert np.all(perm[1:][same] > perm[:-1][same])


def test_counting_sort_edge_cases(orc):
    assert len(orc.counting_sort(np.zeros(0, np.int32), 4)) == 0
    assert np.array_equal(orc.counting_sort(np.array([3, 3, 3], np.int32), 4), [0, 1, 2])
    assert np.array_equal(orc.counting_sort(np.array([2, 0, 1, 0], np.int32), 3), [1, 3, 2, 0])


def _c0_params(orc, g):
    X, Y, Z = (int(a) for a in g["domain"])
    p = phys_params(orc.reference_params(X, Y, Z))
    return p


def test_reference_params_match_reference_init(orc):
    g = golden("ref_c0_step.npz")
    p = _c0_params(orc, g)
    assert list(p.grid) == list(g["grid"])
    f = g["floats"]  # kernelRadius, cell_size, cubic_k, cubic_l, kernelFactor, particleRadius
    assert p.kernel_radius == f[0] and p.cell_size == f[1]
    assert np.float32(p.cubic_k) == f[2] and np.float32(p.cubic_l) == f[3]
    assert p.kernel_factor == f[4] and p.particle_radius == f[5]


def test_compat_step_bit_exact_c0(orc):
    g = golden("ref_c0_step.npz")
    p = _c0_params(orc, g)
    o = orc.compat_step(p, float(g["dt"]), g["x0"], g["v0"], cap=256)
    n = len(g["x0"])
    # neighbour lists: same sets and the same order as the reference
    ref_off, ref_nbr = g["nbr_off"], g["nbr"]
    assert np.array_equal(np.diff(ref_off), o["nbr_count"])
    flat = np.concatenate([o["nbr_idx"][i, :o["nbr_count"][i]] for i in range(n)])
    assert np.array_equal(flat, ref_nbr)
    assert np.array_equal(o["lambdas"][:n], g["lam"])
    assert np.array_equal(o["xs"], g["xs"])
    assert np.array_equal(o["x"], g["x"])
    assert np.array_equal(o["v"], g["v"])


def test_compat_step_bit_exact_with_solids_two_steps(orc):
    g = golden("ref_solids_2step.npz")
    X, Y, Z = (int(a) for a in g["domain"])
    p = phys_params(orc.reference_params(X, Y, Z))
    n = len(g["x0"])
    o1 = orc.compat_step(p, float(g["dt"]), g["x0"], g["v0"], solid=g["solid"], cap=256)
    assert [list(a) for a in rows_sets(o1["nbr_count"], o1["nbr_idx"])] == \
        [list(a) for a in csr_sets(g["nbr_off1"], g["nbr1"])]
    assert (g["nbr1"] >= n).sum() > 0, "fixture must contain solid neighbours"
    assert np.array_equal(o1["lambdas"][:n], g["lam1"])
    assert np.array_equal(o1["x"], g["x1"]) and np.array_equal(o1["v"], g["v1"])
    o2 = orc.compat_step(p, float(g["dt"]), o1["x"], o1["v"], solid=g["solid"],
                         lambdas=o1["lambdas"], cap=256)
    assert np.array_equal(o2["lambdas"][:n], g["lam2"])
    assert np.array_equal(o2["x"], g["x2"]) and np.array_equal(o2["v"], g["v2"])


def test_jacobi_changes_only_the_position_pass(orc):
    g = golden("ref_c0_step.npz")
    p = _c0_params(orc, g)
    p.jacobi = 1
    o = orc.compat_step(p, float(g["dt"]), g["x0"], g["v0"], cap=256)
    n = len(g["x0"])
    assert np.array_equal(o["lambdas"][:n], g["lam"])          # lambda pass unchanged
    assert np.array_equal(np.diff(g["nbr_off"]), o["nbr_count"])
    assert not np.array_equal(o["x"], g["x"])                   # Gauss-Seidel differs


def test_compat_cell_range_error_without_clamp(orc):
    p = phys_params(orc.reference_params(8, 8, 8))
    x = np.array([[4.0, 4.0, 4.0], [100.0, 4.0, 4.0]], np.float32)
    with pytest.raises(RuntimeError):
        orc.compat_step(p, 0.01, x, np.zeros_like(x))
    p.clamp_cells = 1
    o = orc.compat_step(p, 0.01, x, np.zeros_like(x))
    assert np.isfinite(o["x"]).all()


def test_pbf_oracle_float_vs_double(orc):
    from lustrine_gb300 import scenes
    sc = scenes.config0(seed=3)
    p = orc.reference_params(*sc.domain)
    phys_params(p)
    p.iterations = 4
    p.c_xsph = 0.01
    v = np.zeros_like(sc.x)
    d = orc.pbf_step(p, sc.dt, sc.x, v, dtype=np.float64)
    f = orc.pbf_step(p, sc.dt, sc.x, v, dtype=np.float32)
    assert np.abs(d["x"] - f["x"]).max() < 1e-4
    assert np.abs(d["density"] - f["density"]).max() / np.abs(d["density"]).max() < 1e-5


def test_pbf_oracle_conserves_mass_and_stays_in_box(orc):
    from lustrine_gb300 import scenes
    sc = scenes.config0(seed=4)
    p = phys_params(orc.reference_params(*sc.domain))
    p.iterations = 4
    x, v = sc.x.astype(np.float64), np.zeros((sc.n, 3))
    for _ in range(5):
        r = orc.pbf_step(p, sc.dt, x, v)
        x, v = r["x"], r["v"]
    assert np.isfinite(x).all()
    assert (x >= 0.5 - 1e-9).all() and (x <= 39.5 + 1e-9).all()
    # density of the FP64 helper equals the step's last lambda pass at the same state
    rho = orc.pbf_density(p, x)
    assert rho.shape == (sc.n,) and (rho > 0).all()


def test_sand_step_bit_exact_five_steps(orc):
    """simulate_sand restated (integration with attract and blow, the stable
    sort that permutes the state, symmetric lists, 4 contact/friction
    substeps) equals the reference's five calls bit for bit, lists in the
    reference's push order."""
    g = golden("ref_sand_steps.npz")
    X, Y, Z = (int(a) for a in g["domain"])
    p = phys_params(orc.reference_params(X, Y, Z))
    n = len(g["x0"])
    x, v, att = g["x0"], g["v0"], np.zeros(n, np.int32)
    prev = False
    for k in range(len(g["attract"])):
        s = k + 1
        ctl = orc.sand_controls(player=g["player"][k], attract=bool(g["attract"][k]), blow=bool(g["blow"][k]),
                                prev_attract=prev, diameter=float(g["diameter"]))
        o = orc.sand_step(p, ctl, float(g["dt"]), x, v, att, solid=g["solid"], cap=96)
        off, flat = g[f"nbr_off{s}"], g[f"nbr{s}"]
        assert np.array_equal(np.diff(off), o["nbr_count"])
        assert np.array_equal(np.concatenate([o["nbr_idx"][i, :o["nbr_count"][i]] for i in range(n)]), flat)
        assert np.array_equal(o["x"], g[f"x{s}"]) and np.array_equal(o["v"], g[f"v{s}"])
        assert np.array_equal(o["attracted"], g[f"att{s}"])
        x, v, att = o["x"], o["v"], o["attracted"]
        prev = bool(g["attract"][k])
    # the fixture exercises static neighbours and the attract flags
    assert (g["nbr5"] >= n).sum() > 0 and g["att2"].sum() > 0 and g["att4"].sum() == 0
