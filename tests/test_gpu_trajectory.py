"""FP64 GPU trajectories against the reference at the benchmark configurations' own sizes.

* sphere_traj_n10648: the basalt sphere of 10,000 requested particles (10,648 on the HCP lattice, h = 1.3 x the
  lattice spacing), Tillotson, ContinuityEquation + PressureForce + StandardAV, Barnes-Hut theta 0.5 octupole,
  predictor-corrector with the Courant criterion, 100 steps (the reference: core/timestepping/
  TimeStepping.cpp:272-346 over core/sph/solvers/SymmetricSolver.cpp:109-141 and GravitySolver.cpp:64-91).
* impact_traj_n217823: the solid impact of 200,000 + 5,000 requested particles (217,823), Hooke + von Mises +
  Grady-Kipp with the reference's own flaws, SolidStressForce, adaptive h, its first 10 steps.

Both runs are the reference's (oracle/ref_driver.cpp, SEQUENTIAL scheduler). Tolerances: one derivative
evaluation within 1e-12 and every dumped state within 1e-10 of each quantity's maximum magnitude over all
particles; the sums over all particles within 1e-10 of sqrt(N * sum of squares); per particle, density,
smoothing length, specific energy and |v| (where bounded away from zero) within 1e-9 relative; the time steps
within 1e-10; the integrals (core/physics/Integrals.cpp:24-91), also in a rotating frame, within 3e-11, the
rounding bound N eps of the reference's own uncompensated sums over 217,823 particles.
"""
import numpy as np
import pytest

import cases
import trajectory
from opensph_gb300.solver import GpuSolver

pytestmark = pytest.mark.gpu

TOL_EVAL = 1e-12
TOL_STATE = 1e-10
TOL_SUM = 1e-10
TOL_PARTICLE = 1e-9
TOL_INTEGRAL = 3e-11

FIXTURES = ["sphere_traj_n10648", "impact_traj_n217823"]
STATE = ["r", "v", "dv", "rho", "drho", "u", "du", "p", "cs", "S", "dS", "D", "dD"]


@pytest.fixture(scope="module", params=FIXTURES)
def fx(request):
    return cases.load(request.param)


def test_derivatives_match_reference(fx):
    cfg, keep = cases.config_of(fx)
    with GpuSolver(cfg, keep) as g:
        g.set_state(cases.state_of(fx, "s0_"))
        g.integrate()
        got = g.get_state()
    errs = trajectory.sampled_errors(fx, "d0_", got, ["dv", "drho", "du", "p", "cs", "dS", "dD"])
    assert errs, "fixture without derivatives"
    for f, (e, es) in errs.items():
        assert e < TOL_EVAL, (f, e)
        assert es < TOL_SUM, (f, es)
    idx = fx["sample_idx"].astype(np.int64)
    if "d0_ncnt" in fx:
        np.testing.assert_array_equal(got["ncnt"][idx], fx["d0_ncnt"])
        assert int(got["ncnt"].sum()) == int(fx["d0_ncnt@sum"][0])


def test_trajectory_matches_reference(fx):
    cfg, keep = cases.config_of(fx)
    dumped = [int(k) for k in fx["dumped_steps"]]
    report = []
    with GpuSolver(cfg, keep) as g:
        g.set_state(cases.state_of(fx, "s0_"))
        g.timestep = float(fx["dts"][0])
        dts = []
        done = 0
        for k in dumped:
            for _ in range(k - done):
                g.step(1)
                dts.append(g.timestep)
            done = k
            got = g.get_state()
            pre = f"t{k}_"
            for f, (e, es) in trajectory.sampled_errors(fx, pre, got, STATE).items():
                report.append((k, f, e, es))
                assert e < TOL_STATE, (k, f, e)
                assert es < TOL_SUM, (k, f, es)
            for f, e in trajectory.per_particle_errors(fx, pre, got).items():
                assert e < TOL_PARTICLE, (k, "per particle", f, e)
            ints = trajectory.integral_errors(fx, pre, g.totals(), g.totals(trajectory.FRAME_OMEGA))
            for f, e in ints.items():
                assert e < TOL_INTEGRAL, (k, f, e)
    np.testing.assert_allclose(dts, fx["dts"][1:len(dts) + 1], rtol=1e-10)
    worst = max(report, key=lambda t: t[2])
    print(f"worst sampled error {worst[2]:.2e} ({worst[1]} after {worst[0]} steps)")


def test_initial_integrals_match_reference(fx):
    cfg, keep = cases.config_of(fx)
    with GpuSolver(cfg, keep) as g:
        g.set_state(cases.state_of(fx, "s0_"))
        ints = trajectory.integral_errors(fx, "s0_", g.totals(), g.totals(trajectory.FRAME_OMEGA))
        tot = g.totals()
    for f, e in ints.items():
        assert e < TOL_INTEGRAL, (f, e)
    assert abs(tot[6] - float(fx["s0_kinetic_energy"][0])) <= TOL_INTEGRAL * abs(float(fx["s0_energy"][0]))
    assert abs(tot[7] - float(fx["s0_internal_energy"][0])) <= TOL_INTEGRAL * abs(float(fx["s0_energy"][0]))
