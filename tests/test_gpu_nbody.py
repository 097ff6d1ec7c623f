"""GPU HardSphereSolver (sphgpu_collide / sphgpu_step with the N-body solver) against the CPU oracle and the
reference's golden runs and N-body test scenarios (core/gravity/test/NBodySolver.cpp).

Decisions (which pairs collide, in which order, which merge) must be identical; states agree to the rounding
of the Barnes-Hut sums and of cbrt (the radius of a merger), amplified over the fixture's steps."""
import numpy as np
import pytest

import nbody_cases as nc
from oracle import oracle
from opensph_gb300 import abi
from opensph_gb300.solver import GpuSolver, SphGpuError

pytestmark = pytest.mark.gpu

# relative to the largest magnitude of each field
TOL_RUN = 1e-10
TOL_CALL = 1e-13


def gpu_run(cfg, keep, st, steps, dt, per_step=False):
    with GpuSolver(cfg, keep) as g:
        g.set_state(st)
        g.timestep = dt
        counts = []
        if per_step:
            for _ in range(steps):
                g.step(1)
                counts.append(g.n)
        else:
            g.step(steps)
        out = g.get_state(nc.FIELDS)
        return out, g.collision_stats(), g.n, g.timestep, counts


@pytest.mark.parametrize("name", nc.FIXTURES)
def test_gpu_run_matches_oracle_and_reference(name):
    fx = nc.load(name)
    cfg, keep = nc.config_of(fx)
    steps = nc.steps_of(fx)
    dt0 = float(fx["dts"][0])
    got, stats, n, dt_next, counts = gpu_run(cfg, keep, nc.state_of(fx, "s0_"), steps, dt0, per_step=True)
    ref = nc.state_of(fx, "s0_")
    ora_dt, _, ora_counts, ora_stats, _ = oracle.nbody_run(cfg, ref, steps, dt0)
    assert stats == [int(x) for x in ora_stats]
    assert stats == [int(x) for x in fx["collision_stats"]]
    assert counts == [int(x) for x in ora_counts] == [int(x) for x in fx["counts"]]
    assert abs(dt_next - ora_dt) <= 1e-12 * ora_dt
    for f in nc.FIELDS:
        assert nc.scale_err(got[f], ref[f]) < TOL_RUN, f
        assert nc.scale_err(got[f], fx["sN_" + f]) < TOL_RUN, f


@pytest.mark.parametrize("name", nc.FIXTURES)
def test_gpu_single_collide_matches_oracle(name):
    fx = nc.load(name)
    cfg, keep = nc.config_of(fx)
    st = nc.state_of(fx, "s0_")
    dt = 0.5 * float(fx["dts"][0])
    with GpuSolver(cfg, keep) as g:
        g.set_state(st)
        g.collide(dt)
        got = g.get_state(nc.FIELDS)
        stats = g.collision_stats()
    ref = nc.state_of(fx, "s0_")
    ora_stats, _ = oracle.nbody_collide(cfg, ref, dt, prev_removed=[])
    assert stats == [int(x) for x in ora_stats]
    assert len(got["m"]) == len(ref["m"])
    for f in nc.FIELDS:
        assert nc.scale_err(got[f], ref[f]) < TOL_CALL, f


def test_gpu_take_removed_lists_the_merged_particles():
    fx = nc.load("nbody_merge_n1000")
    cfg, keep = nc.config_of(fx)
    dt = 150.0
    with GpuSolver(cfg, keep) as g:
        g.set_state(nc.state_of(fx, "s0_"))
        g.collide(dt)
        removed = g.take_removed()
        again = g.take_removed()
        n = g.n
    ref = nc.state_of(fx, "s0_")
    _, _, origin = oracle.nbody_collide(cfg, ref, dt, origin=True, prev_removed=[])
    expected = np.setdiff1d(np.arange(len(fx["s0_m"])), origin)
    assert len(expected) > 0
    np.testing.assert_array_equal(removed, expected)
    assert len(again) == 0 and n == len(origin)


def test_gpu_removed_indices_persist_to_the_next_call():
    # two collide calls: the second call's first pass skips the indices the first call removed
    fx = nc.load("nbody_merge_n1000")
    cfg, keep = nc.config_of(fx)
    st = nc.state_of(fx, "s0_")
    with GpuSolver(cfg, keep) as g:
        g.set_state(st)
        for _ in range(4):
            g.collide(150.0)
        got = g.get_state(nc.FIELDS)
        stats = g.collision_stats()
    ref = nc.state_of(fx, "s0_")
    prev = []
    total = np.zeros(4, dtype=np.uint64)
    for _ in range(4):
        s, _ = oracle.nbody_collide(cfg, ref, 150.0, prev_removed=prev)
        total += s
    assert stats == [int(x) for x in total]
    for f in nc.FIELDS:
        assert nc.scale_err(got[f], ref[f]) < TOL_CALL, f


def test_gpu_integrate_is_self_gravity_with_h_derivatives_zeroed():
    fx = nc.load("nbody_bounce_n1000")
    cfg, keep = nc.config_of(fx)
    st = nc.state_of(fx, "s0_")
    st["v"].reshape(-1, 4)[:, 3] = 0.25
    with GpuSolver(cfg, keep) as g:
        g.set_state(st)
        g.integrate()
        got = g.get_state(["dv", "v"])
    ref = dict(st)
    oracle.nbody_integrate(cfg, ref)
    assert nc.scale_err(got["dv"], ref["dv"]) < 1e-14
    np.testing.assert_array_equal(got["dv"].reshape(-1, 4)[:, 3], 0.0)
    np.testing.assert_array_equal(got["v"].reshape(-1, 4)[:, 3], 0.0)


def test_gpu_mixed_precision_walk_keeps_the_events():
    fx = nc.load("nbody_bounce_n1000")
    cfg, keep = nc.config_of(fx, precision=abi.PRECISION_MIXED)
    got, stats, n, _, _ = gpu_run(cfg, keep, nc.state_of(fx, "s0_"), 2, float(fx["dts"][0]))
    ref = nc.state_of(fx, "s0_")
    cfg64, keep64 = nc.config_of(fx)
    _, _, _, ora_stats, _ = oracle.nbody_run(cfg64, ref, 2, float(fx["dts"][0]))
    assert stats == [int(x) for x in ora_stats]
    assert nc.scale_err(got["dv"], ref["dv"]) < 2e-6
    assert nc.scale_err(got["r"], ref["r"]) < 1e-9


def _kat(cfg, keep, st, steps=10000, dt=1e-4):
    with GpuSolver(cfg, keep) as g:
        g.set_state(st)
        g.timestep = dt
        g.step(steps)
        return g.get_state(nc.FIELDS), g.collision_stats(), g.n


def test_gpu_two_particles_bounce():
    cfg, keep = nc.kat_config(2, abi.COLLISION_ELASTIC_BOUNCE, restitution_normal=1.0, restitution_tangent=1.0)
    got, stats, n = _kat(cfg, keep, nc.two_particles())
    assert stats == [1, 0, 1, 0] and n == 2
    np.testing.assert_allclose(got["v"].reshape(2, 4)[:, 0], [5.0, -5.0], atol=1e-6)
    ref = nc.two_particles()
    oracle.nbody_run(cfg, ref, 10000, 1e-4)
    for f in nc.FIELDS:
        assert nc.scale_err(got[f], ref[f]) < 1e-12, f


def test_gpu_two_particles_merge_and_off_center():
    cfg, keep = nc.kat_config(2, abi.COLLISION_PERFECT_MERGING, bounce_merge_limit=0.0, rotation_merge_limit=0.0)
    got, stats, n = _kat(cfg, keep, nc.two_particles())
    assert stats == [1, 1, 0, 0] and n == 1
    np.testing.assert_allclose(got["v"][:3], 0.0, atol=1e-6)
    assert got["m"][0] == 4.0
    st = nc.two_particles()
    b = 1.0 + 0.5 - 1e-5
    st["r"][1] = b
    got, stats, n = _kat(cfg, keep, st)
    assert n == 1
    h = got["r"][3]
    L = 0.4 * got["m"][0] * h * h * np.linalg.norm(got["w"][:3])
    assert abs(L - 10.0 * b) < 1e-6 * 10.0 * b


def test_gpu_two_particles_miss_and_rejection():
    st = nc.two_particles()
    st["r"][1] = 1.0 + 0.5 + 1e-5
    cfg, keep = nc.kat_config(2, abi.COLLISION_PERFECT_MERGING, bounce_merge_limit=0.0, rotation_merge_limit=0.0)
    _, stats, n = _kat(cfg, keep, st)
    assert stats == [0, 0, 0, 0] and n == 2
    cfg, keep = nc.kat_config(2, abi.COLLISION_MERGE_OR_BOUNCE, bounce_merge_limit=1e6)
    got, stats, n = _kat(cfg, keep, nc.two_particles())
    assert stats == [1, 0, 1, 0] and n == 2
    np.testing.assert_array_equal(got["m"], [2.0, 2.0])


def test_gpu_repel_overlap():
    st = {"r": np.array([0.0, 0.0, 0.0, 1.0, 1.0, 0.0, 0.0, 0.25]), "v": np.array([0.0, 0, 0, 0, -1e-3, 0, 0, 0]),
          "dv": np.zeros(8), "m": np.array([1.0, 0.1]), "w": np.zeros(8)}
    cfg, keep = nc.kat_config(2, abi.COLLISION_ELASTIC_BOUNCE, abi.OVERLAP_REPEL, restitution_normal=0.0,
                              restitution_tangent=0.0)
    with GpuSolver(cfg, keep) as g:
        g.set_state(st)
        g.collide(1e-4)
        got = g.get_state(nc.FIELDS)
        assert g.collision_stats() == [0, 0, 0, 1]
    r = got["r"].reshape(2, 4)
    assert abs((r[0, 0] * 1.0 + r[1, 0] * 0.1) / 1.1 - 0.1 / 1.1) < 1e-12
    assert abs(np.linalg.norm(r[0, :3] - r[1, :3]) - 1.25) < 1e-12


@pytest.mark.parametrize("handler,overlap,check", [
    (abi.COLLISION_PERFECT_MERGING, abi.OVERLAP_FORCE_MERGE, lambda n, n0: n == 1),
    (abi.COLLISION_MERGE_OR_BOUNCE, abi.OVERLAP_REPEL, lambda n, n0: 1 < n < 30),
    (abi.COLLISION_ELASTIC_BOUNCE, abi.OVERLAP_NONE, lambda n, n0: n == n0),
])
def test_gpu_cloud_scenarios_match_oracle(handler, overlap, check):
    st = nc.cloud()
    n0 = len(st["m"])
    cfg, keep = nc.kat_config(n0, handler, overlap, bounce_merge_limit=0.0, rotation_merge_limit=0.0)
    got, stats, n = _kat(cfg, keep, nc.cloud())
    assert check(n, n0)
    ref = nc.cloud()
    _, _, counts, ora_stats, _ = oracle.nbody_run(cfg, ref, 10000, 1e-4)
    assert stats == [int(x) for x in ora_stats]
    assert n == counts[-1]
    for f in ("r", "v", "dv", "m"):
        assert nc.scale_err(got[f], ref[f]) < 1e-9, f
    # the spins of a symmetric cloud are rounding noise: compare them on the spin scale |v| / h = 400 / s
    assert np.abs(got["w"] - ref["w"]).max() < 1e-9 * 400.0


def test_gpu_no_handler_ignores_collisions_and_sph_calls_are_refused():
    st = nc.two_particles()
    cfg, keep = nc.kat_config(2, abi.COLLISION_NONE)
    got, stats, n = _kat(cfg, keep, st, steps=10000)
    assert stats == [0, 0, 0, 0] and n == 2
    np.testing.assert_allclose(got["v"].reshape(2, 4)[:, 0], [-5.0, 5.0])
    with GpuSolver(cfg, keep) as g:
        with pytest.raises(SphGpuError) as e:
            g.pairs()
        assert e.value.code == abi.ERR_UNSUPPORTED


def test_gpu_collision_work_space_overflow_keeps_a_consistent_state():
    # a collide call whose loop runs out of collision records returns SPHGPU_ERR_CAPACITY with the collisions it
    # processed applied and the particles they merged away removed: mass and momentum are conserved and the
    # particle count drops by the mergers counted
    st = nc.cloud()
    n0 = len(st["m"])
    cfg, keep = nc.kat_config(n0, abi.COLLISION_PERFECT_MERGING, abi.OVERLAP_FORCE_MERGE, bounce_merge_limit=0.0,
                              rotation_merge_limit=0.0, collision_records=4)
    m0 = float(np.sum(st["m"]))
    v0 = st["v"].reshape(-1, 4)[:, :3]
    p0 = np.sum(st["m"][:, None] * v0, 0)
    pscale = float(np.sum(st["m"] * np.linalg.norm(v0, axis=1)))
    with GpuSolver(cfg, keep) as g:
        g.set_state(nc.cloud())
        with pytest.raises(SphGpuError) as e:
            g.collide(0.3)  # every sphere meets the others at the centre at t = 0.25
        assert e.value.code == abi.ERR_CAPACITY
        g._refresh_count()
        stats = g.collision_stats()
        got = g.get_state(nc.FIELDS)
        n = g.n
    assert stats[1] > 0 and n == n0 - stats[1]
    assert abs(float(np.sum(got["m"])) - m0) <= 1e-12 * m0
    p = np.sum(got["m"][:, None] * got["v"].reshape(-1, 4)[:, :3], 0)
    assert np.max(np.abs(p - p0)) <= 1e-12 * pscale
