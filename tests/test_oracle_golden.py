"""Pins the CPU oracle (oracle/) to golden vectors produced by the reference itself (tests/golden/).

These mirror the reference's own tests of the path: Tillotson values (core/physics/test/Eos.cpp:20-55),
finder vs brute force (core/objects/finders/test/Finders.cpp:55-157), Barnes-Hut vs brute force and the
6-particle known answer (core/gravity/test/BarnesHut.cpp:23-158), kernel values
(core/sph/kernel/test/Kernel.cpp:134-177), and whole solver steps through the reference's library entry.
"""
import numpy as np
import pytest

import cases
from opensph_gb300 import abi
from oracle import oracle

# Sums over neighbours are taken in a different order than the reference's sequential scatter, so the
# derivatives agree to rounding: bound 1e-12 of each quantity's magnitude for one evaluation, 1e-10 after
# the fixture's steps (the FP64 parity bound).
TOL_EVAL = 1e-12
TOL_STEPS = 1e-10


def test_tillotson_known_values():
    # core/physics/test/Eos.cpp:20-55 (rho0 = 2.7, u0 = 1e5), rel. 1e-6
    m = abi.basalt(density=2.7, tillotson_sublimation=1e5)
    cases_ = [((2.7, 1e5), (337500.0, 99444.4453)), ((2.0, 1e5), (-5.12736563e9, 54744.2812)),
              ((2.0, 1e10), (9.34812365e9, 67291.1719)), ((2.8, 1e10), (1.50259651e10, 135296.312)),
              ((2.6, 1e7), (-883133952.0, 88856.2188)), ((2.7, 1e7), (13900990.0, 99483.1953)),
              ((2.8, 1e7), (1.03996064e9, 103983.867))]
    rho = np.array([c[0][0] for c in cases_])
    u = np.array([c[0][1] for c in cases_])
    p, cs = oracle.eos(m, rho, u)
    for k, (_, (pe, ce)) in enumerate(cases_):
        assert p[k] == pytest.approx(pe, rel=1e-6)
        assert cs[k] == pytest.approx(ce, rel=1e-6)


def test_tillotson_grid_bit_exact():
    fx = cases.load("eos_tillotson")
    m = abi.basalt(density=2.7, tillotson_sublimation=1e5)
    p, cs = oracle.eos(m, fx["rho"], fx["u"])
    np.testing.assert_array_equal(p, fx["p"])
    np.testing.assert_array_equal(cs, fx["cs"])


def test_cubic_spline_kernel_values():
    # core/sph/kernel/test/Kernel.cpp:134-177: W(0) = 1/pi, W(1) = 1/(4 pi), grad W(1) = -3/(4 pi)
    w, g, _ = oracle.kernel_values([0.0, 1.0, 4.0])
    assert w[0] == pytest.approx(1 / np.pi, rel=1e-6)
    assert w[1] == pytest.approx(0.25 / np.pi, rel=1e-6)
    assert g[1] == pytest.approx(-0.75 / np.pi, rel=1e-6)
    assert w[2] == 0.0 and g[2] == 0.0
    # LUT normalisation: integral of W over the support is 1
    q = np.linspace(0.0, 2.0, 20001)
    wq, _, _ = oracle.kernel_values(q * q)
    integral = np.trapezoid(4 * np.pi * q * q * wq, q)
    assert integral == pytest.approx(1.0, abs=1e-4)


def test_pair_set_matches_reference_kdtree():
    fx = cases.load("pairs_n1500")
    pi, pj = oracle.pairs(fx["r"])
    mine = set(zip(pi.tolist(), pj.tolist()))
    ref = {(min(i, j), max(i, j)) for i, j in zip(fx["pair_i"].tolist(), fx["pair_j"].tolist())}
    assert mine == ref


def test_pairs_empty_and_single():
    pi, pj = oracle.pairs(np.zeros(0))
    assert pi.size == 0
    pi, pj = oracle.pairs(np.array([0.0, 0.0, 0.0, 1.0]))
    assert pi.size == 0


@pytest.mark.parametrize("name", ["gravity_n3000", "gravity_n3000_t07"])
def test_barnes_hut_matches_reference(name):
    fx = cases.load(name)
    theta = float(str(fx["driver_args"]).split()[2])
    dv, stats = oracle.gravity_bh(fx["r"], fx["m"], G=1.0, theta=theta)
    # identical tree: same node count and the same number of approximated / exact interactions
    assert stats == [int(fx["nodes_approx"][0]), int(fx["nodes_exact"][0]), int(fx["node_count"][0])]
    assert cases.scale_err(cases.vec3(dv), cases.vec3(fx["a_bh"])) < 1e-13
    ad = oracle.gravity_direct(fx["r"], fx["m"], G=1.0)
    assert cases.scale_err(cases.vec3(ad), cases.vec3(fx["a_direct"])) < 1e-14


def test_barnes_hut_six_particle_known_answer():
    # core/gravity/test/BarnesHut.cpp:23-45, 138-158: point masses, leaf size 1, theta 0.5
    r = np.array([[2, 3, 0, 1], [5, 4, 0, 1], [9, 6, 0, 1], [4, 7, 0, 1], [8, 1, 0, 1], [7, 2, 0, 1]], "f8")
    m = np.ones(6)
    expected = np.array([0.020169998934707004, -0.007912678499211458, 0.0])
    for order, eps in [(0, 4e-4), (2, 8e-5), (3, 1e-5)]:
        a = oracle.gravity_points(r.ravel(), m, np.array([-10.0, 10.0, 0.0, 1.0]), G=1.0, theta=0.5,
                                  order=order, leaf_size=1, kernel_radius=0)
        assert not np.array_equal(a[:3], expected)
        # almostEqual on vectors (core/objects/geometry/Vector.h:675-677)
        d2 = np.sum((a[:3] - expected) ** 2)
        assert d2 <= eps * eps * (1.0 + max(np.sum(a[:3] ** 2), np.sum(expected ** 2)))


def test_barnes_hut_small_theta_is_brute_force():
    # core/gravity/test/BarnesHut.cpp:47-80
    fx = cases.load("gravity_n3000")
    dv, _ = oracle.gravity_bh(fx["r"], fx["m"], G=1.0, theta=1e-6)
    assert cases.scale_err(cases.vec3(dv), cases.vec3(fx["a_direct"])) < 1e-13


@pytest.mark.parametrize("name", ["sphere_n1000", "impact_n1200", "gas_n1500", "impact_asym_n1200"])
def test_integrate_matches_reference(name):
    fx = cases.load(name)
    cfg, keep = cases.config_of(fx)
    st = cases.state_of(fx, "s0_")
    oracle.integrate(cfg, st)
    for f in ["dv", "drho", "du", "divv", "p", "cs", "gradv", "dS", "dD", "reduce", "S", "corr"]:
        if "d0_" + f in fx:
            assert cases.scale_err(st[f], fx["d0_" + f]) < TOL_EVAL, f
    np.testing.assert_array_equal(st["ncnt"], fx["d0_ncnt"])


@pytest.mark.parametrize("name", ["sphere_n1000", "impact_n1200", "gas_n1500", "impact_all_n1200",
                                  "gas_all_n1500", "impact_asym_n1200", "sphere_cached_n1000"])
def test_steps_match_reference(name):
    fx = cases.load(name)
    cfg, keep = cases.config_of(fx)
    st = cases.state_of(fx, "s0_")
    steps = len(fx["dts"]) - 1
    dt, dts = oracle.run(cfg, st, steps, float(fx["dts"][0]))
    np.testing.assert_allclose(dts, fx["dts"][:steps], rtol=1e-12)
    assert dt == pytest.approx(float(fx["dts"][steps]), rel=1e-10)
    for f in ["r", "v", "dv", "rho", "drho", "u", "du", "divv", "S", "dS", "D", "dD"]:
        if "sN_" + f in fx:
            assert cases.scale_err(st[f], fx["sN_" + f]) < TOL_STEPS, f


def test_cached_gravity_differs_from_recomputed_gravity():
    # the cached run is not the plain run: the reference reused accelerations between recomputations
    fx = cases.load("sphere_cached_n1000")
    cfg, keep = cases.config_of(fx)
    cfg.gravity_recomputation_period = 0.0
    st = cases.state_of(fx, "s0_")
    oracle.run(cfg, st, len(fx["dts"]) - 1, float(fx["dts"][0]))
    assert cases.scale_err(st["v"], fx["sN_v"]) > 100 * TOL_STEPS


def test_direct_sum_matches_reference_bruteforce_at_65536():
    # BruteForceGravity (core/gravity/BruteForceGravity.h:38-58, 110-129) at N = 65,536: the points regenerate bit
    # for bit from the fixture's seed (sequential sums of the coordinates equal the reference driver's), and the
    # oracle's FP64 direct sum equals the reference's accelerations exactly at 1,024 seeded particles
    fx = cases.load("direct_n65536")
    r, m = cases.direct_points(fx)
    for c in range(3):
        assert np.add.accumulate(r[:, c])[-1] == fx["checksum"][c]
    got = oracle.gravity_direct(r.ravel(), m, G=1.0, targets=fx["sample_idx"]).reshape(-1, 4)
    np.testing.assert_array_equal(got[:, :3], fx["a_direct"].reshape(-1, 4)[:, :3])


def test_attractors_match_reference():
    # BarnesHut::evalAttractors (core/gravity/BarnesHut.cpp:100-125) with two attractors: the particles'
    # accelerations (all four components, as the reference scales the whole separation Vector) and the
    # attractors' accelerations, bit for bit
    fx = cases.load("attractors_n2000")
    dv, acc = oracle.gravity_attractors(fx["r"], fx["m"], fx["attractors"].reshape(-1, 5), fx["a_self"].copy(),
                                        np.zeros(6), G=float(fx["G"][0]))
    np.testing.assert_array_equal(dv, fx["a_total"])
    np.testing.assert_array_equal(acc, fx["attractor_acc"])
