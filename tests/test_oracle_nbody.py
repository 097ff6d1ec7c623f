"""The CPU oracle of HardSphereSolver against the reference: the golden runs of tests/golden/nbody_*.npz
(produced by the reference's own HardSphereSolver + LeapFrog, oracle/ref_driver.cpp) and the scenarios of the
reference's N-body tests (core/gravity/test/NBodySolver.cpp), restated with the inertia tensor off."""
import numpy as np
import pytest

import nbody_cases as nc
from oracle import oracle
from opensph_gb300 import abi


@pytest.mark.parametrize("name", nc.FIXTURES)
def test_oracle_reproduces_reference_run(name):
    fx = nc.load(name)
    cfg, keep = nc.config_of(fx)
    st = nc.state_of(fx, "s0_")
    steps = nc.steps_of(fx)
    dt_next, dts, counts, stats, amb = oracle.nbody_run(cfg, st, steps, float(fx["dts"][0]))
    # every collision, merger, bounce and overlap of the reference, and the same survivors
    np.testing.assert_array_equal(stats, fx["collision_stats"].astype(np.uint64))
    np.testing.assert_array_equal(counts, fx["counts"].astype(np.uint32))
    np.testing.assert_allclose(dts, fx["dts"][:-1], rtol=1e-12)
    assert abs(dt_next - fx["dts"][-1]) <= 1e-12 * fx["dts"][-1]
    # trajectories: the same events; the Barnes-Hut sums differ from the reference's by summation order
    for f in nc.FIELDS:
        assert nc.scale_err(st[f], fx["sN_" + f]) < 1e-12, f


def test_first_step_of_each_fixture_is_exact_up_to_gravity_rounding():
    for name in nc.FIXTURES:
        fx = nc.load(name)
        cfg, keep = nc.config_of(fx)
        st = nc.state_of(fx, "s0_")
        oracle.nbody_run(cfg, st, 1, float(fx["dts"][0]))
        assert len(st["m"]) == len(fx["s1_m"]), name
        np.testing.assert_array_equal(st["m"], fx["s1_m"])
        for f in ("r", "v", "w"):
            assert nc.scale_err(st[f], fx["s1_" + f]) < 1e-14, (name, f)


def _run(cfg, st, steps, dt=1e-4):
    return oracle.nbody_run(cfg, st, steps, dt)


def test_two_particles_bounce():
    # "Collision bounce two": restitution 1, 1 -> the velocities are exchanged, nothing else changes
    st = nc.two_particles()
    cfg, keep = nc.kat_config(2, abi.COLLISION_ELASTIC_BOUNCE, restitution_normal=1.0, restitution_tangent=1.0)
    _, _, counts, stats, _ = _run(cfg, st, 10000)
    assert list(stats) == [1, 0, 1, 0] and counts[-1] == 2
    v = st["v"].reshape(2, 4)
    np.testing.assert_allclose(v[:, 0], [5.0, -5.0], atol=1e-6)
    np.testing.assert_array_equal(st["r"].reshape(2, 4)[:, 3], [1.0, 0.5])
    np.testing.assert_array_equal(st["w"], 0.0)


def test_two_particles_merge():
    # "Collision merge two": perfect merging -> one particle at rest, masses and volumes summed
    st = nc.two_particles()
    cfg, keep = nc.kat_config(2, abi.COLLISION_PERFECT_MERGING, bounce_merge_limit=0.0, rotation_merge_limit=0.0)
    _, _, counts, stats, _ = _run(cfg, st, 10000)
    assert list(stats) == [1, 1, 0, 0] and counts[-1] == 1
    np.testing.assert_allclose(st["v"][:3], 0.0, atol=1e-6)
    assert st["m"][0] == 4.0
    assert abs(st["r"][3] - (1.0 + 0.125) ** (1.0 / 3.0)) < 1e-15
    np.testing.assert_array_equal(st["w"], 0.0)


def test_two_particles_merge_off_center_spins_up():
    # "Collision merge off-center": the merger rotates with the pair's angular momentum m1 m2/(m1+m2) b v
    st = nc.two_particles()
    b = 1.0 + 0.5 - 1e-5
    st["r"][1] = b
    cfg, keep = nc.kat_config(2, abi.COLLISION_PERFECT_MERGING, bounce_merge_limit=0.0, rotation_merge_limit=0.0)
    _, _, counts, stats, _ = _run(cfg, st, 10000)
    assert counts[-1] == 1
    h = st["r"][3]
    L = 0.4 * st["m"][0] * h * h * np.linalg.norm(st["w"][:3])
    assert abs(L - 10.0 * b) < 1e-6 * 10.0 * b


def test_two_particles_merge_miss():
    # "Collision merge miss": offset by more than the sum of radii -> no collision
    st = nc.two_particles()
    st["r"][1] = 1.0 + 0.5 + 1e-5
    cfg, keep = nc.kat_config(2, abi.COLLISION_PERFECT_MERGING, bounce_merge_limit=0.0, rotation_merge_limit=0.0)
    _, _, counts, stats, _ = _run(cfg, st, 10000)
    assert list(stats) == [0, 0, 0, 0] and counts[-1] == 2


def test_two_particles_merge_rejected_bounces():
    # "Collision merge rejection": merge-or-bounce with a large merging limit -> bounce, masses unchanged
    st = nc.two_particles()
    cfg, keep = nc.kat_config(2, abi.COLLISION_MERGE_OR_BOUNCE, bounce_merge_limit=1e6)
    _, _, counts, stats, _ = _run(cfg, st, 10000)
    assert list(stats) == [1, 0, 1, 0] and counts[-1] == 2
    np.testing.assert_array_equal(st["m"], [2.0, 2.0])
    np.testing.assert_array_equal(st["w"], 0.0)


def test_repel_overlap_conserves_centre_of_mass():
    # "Collision repel": two overlapping particles moved apart to touch, centre of mass unchanged
    st = {"r": np.array([0.0, 0.0, 0.0, 1.0, 1.0, 0.0, 0.0, 0.25]), "v": np.array([0.0, 0, 0, 0, -1e-3, 0, 0, 0]),
          "dv": np.zeros(8), "m": np.array([1.0, 0.1]), "w": np.zeros(8)}
    com0 = (st["r"][0] * 1.0 + st["r"][4] * 0.1) / 1.1
    cfg, keep = nc.kat_config(2, abi.COLLISION_ELASTIC_BOUNCE, abi.OVERLAP_REPEL, restitution_normal=0.0,
                              restitution_tangent=0.0)
    stats, _ = oracle.nbody_collide(cfg, st, 1e-4)
    assert list(stats) == [0, 0, 0, 1]
    r = st["r"].reshape(2, 4)
    assert abs((r[0, 0] * 1.0 + r[1, 0] * 0.1) / 1.1 - com0) < 1e-12
    assert abs(np.linalg.norm(r[0, :3] - r[1, :3]) - 1.25) < 1e-12


def test_cloud_merges_into_one():
    # "Collision cloud merge": particles fired into one point all merge
    st = nc.cloud()
    n = len(st["m"])
    cfg, keep = nc.kat_config(n, abi.COLLISION_PERFECT_MERGING, abi.OVERLAP_FORCE_MERGE, bounce_merge_limit=0.0,
                              rotation_merge_limit=0.0)
    m0 = st["m"].sum()
    _, _, counts, stats, _ = _run(cfg, st, 10000)
    assert counts[-1] == 1
    assert abs(st["m"][0] - m0) < 1e-12 * m0


def test_cloud_merge_and_bounce():
    # "Collision cloud merge&bounce": with repelled overlaps some particles bounce away
    st = nc.cloud()
    n = len(st["m"])
    cfg, keep = nc.kat_config(n, abi.COLLISION_MERGE_OR_BOUNCE, abi.OVERLAP_REPEL, bounce_merge_limit=0.0,
                              rotation_merge_limit=0.0)
    _, _, counts, _, _ = _run(cfg, st, 10000)
    assert 1 < counts[-1] < 30


def test_cloud_bounce_keeps_every_particle():
    # "Collision cloud bounce": elastic bounces only, no overlaps, no particle lost
    st = nc.cloud()
    n = len(st["m"])
    cfg, keep = nc.kat_config(n, abi.COLLISION_ELASTIC_BOUNCE, abi.OVERLAP_NONE)
    _, _, counts, stats, _ = _run(cfg, st, 10000)
    assert counts[-1] == n and stats[0] > 0 and stats[1] == 0


def test_removed_indices_of_the_previous_call_are_skipped_by_the_next_first_pass():
    # the reference clears its removed set only after the first pass of the next collide call
    fx = nc.load("nbody_merge_n1000")
    cfg, keep = nc.config_of(fx)
    a = nc.state_of(fx, "s0_")
    b = nc.state_of(fx, "s0_")
    prev = list(range(0, 1000, 3))
    sa, _ = oracle.nbody_collide(cfg, a, 50.0, prev_removed=[])
    sb, _ = oracle.nbody_collide(cfg, b, 50.0, prev_removed=prev)
    assert sb[0] < sa[0]
