"""The CPU oracle against the reference's trajectories at the benchmark configurations' sizes (CPU only).

The fixtures are the reference's own runs (tests/golden/make_golden.py): the 10,648-particle basalt sphere over
100 steps and the 217,823-particle solid impact over its first 10 steps. The oracle restates the reference's
algorithms, so it follows both trajectories to rounding: within 1e-10 of each quantity's maximum magnitude at
every dump, with the reference's time steps within 1e-10, and its totals (Neumaier-compensated sums) within
1e-12 of the reference's integrals of the initial states (core/physics/Integrals.cpp:24-91).
"""
import numpy as np
import pytest

import cases
import trajectory
from oracle import oracle

TOL_STATE = 1e-10


@pytest.mark.parametrize("name", ["sphere_traj_n10648", "impact_traj_n217823"])
def test_oracle_follows_reference_trajectory(name):
    fx = cases.load(name)
    cfg, _ = cases.config_of(fx)
    st = cases.state_of(fx, "s0_")
    dt = float(fx["dts"][0])
    done = 0
    for k in (int(x) for x in fx["dumped_steps"]):
        dt, _ = oracle.run(cfg, st, k - done, dt)
        done = k
        errs = trajectory.sampled_errors(fx, f"t{k}_", st, ["r", "v", "dv", "rho", "u", "S", "D"])
        for f, (e, _) in errs.items():
            assert e < TOL_STATE, (k, f, e)
        np.testing.assert_allclose(dt, fx["dts"][k], rtol=1e-10)


@pytest.mark.parametrize("name", ["sphere_traj_n10648", "impact_traj_n217823"])
def test_oracle_totals_match_reference_integrals(name):
    fx = cases.load(name)
    st = cases.state_of(fx, "s0_")
    tot = oracle.totals(st)
    for f, e in trajectory.integral_errors(fx, "s0_", tot).items():
        assert e < 1e-12, (f, e)
