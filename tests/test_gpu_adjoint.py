"""The adjoint of the frozen-list hydrodynamic step (sphgpu_adjoint_forward / sphgpu_adjoint_backward).

Checks, on a 2,231-particle gas impact (20 leap-frog steps, lists rebuilt and checkpoints every 5 steps):
* the FP64 forward loss against the oracle's restatement of the same model;
* the FP64 gradient against the oracle's FP64 tangent-linear (dual-number) run, in seeded per-particle
  directions of every input (relative 1e-9: both are exact derivatives, only rounding differs);
* the FP64 and mixed gradients against FP64 central finite differences in 8 seeded smooth directions
  (relative 1e-4);
* recomputation between checkpoints does not change the result (checkpoint interval 1 vs 5, bit for bit);
* the thin torch.autograd.Function harness around the C ABI pair gives the same gradients;
* argument and call-order errors.
"""
import numpy as np
import pytest

import adjoint_cases as ac
from opensph_gb300 import abi
from opensph_gb300.solver import SphGpuError
from oracle import oracle

pytestmark = pytest.mark.gpu

TOL_TANGENT = 1e-9
TOL_FD = 1e-4
FD_EPS = 1e-6


@pytest.fixture(scope="module")
def case():
    st, nt = ac.gas_state()
    return st, nt


def oracle_loss(st, nt, t=None, steps=ac.STEPS, rebuild=ac.REBUILD, alpha=1.5):
    return oracle.frozen_loss(st["r"], st["v"], st["m"], st["rho"], st["u"], steps, ac.DT, nt,
                              rebuild_every=rebuild, alpha=alpha, tangent=t)


def test_forward_loss_matches_oracle(case):
    st, nt = case
    ref, _ = oracle_loss(st, nt)
    with ac.solver_for(st) as g:
        loss = g.adjoint_forward(ac.config(nt))
        # the handle's state is not changed by the adjoint run
        np.testing.assert_array_equal(g.get_quantity(abi.Q_POSITION, 1), st["v"])
    # same pair terms in the same order; only the final sum over particles runs in another order
    assert abs(loss - ref) <= 1e-13 * abs(ref)


def test_gradient_matches_tangent_linear_fp64(case):
    st, nt = case
    n = len(st["m"])
    rng = np.random.default_rng(11)
    with ac.solver_for(st) as g:
        g.adjoint_forward(ac.config(nt))
        grad = g.adjoint_backward()
    for _ in range(4):
        t = ac.rough_direction(rng, n)
        _, ref = oracle_loss(st, nt, t)
        mine = ac.dot(grad, t)
        assert abs(mine - ref) <= TOL_TANGENT * abs(ref), (mine, ref)
    # the AV alpha on its own
    _, ref = oracle_loss(st, nt, {"alpha": 1.0})
    assert abs(grad["alpha"] - ref) <= TOL_TANGENT * abs(ref)


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_MIXED], ids=["fp64", "mixed"])
def test_gradient_matches_central_differences(case, precision):
    st, nt = case
    rng = np.random.default_rng(5)
    with ac.solver_for(st) as g:
        g.adjoint_forward(ac.config(nt, precision=precision))
        grad = g.adjoint_backward()
    worst = 0.0
    for _ in range(8):
        t = ac.smooth_direction(rng, st, nt)
        vals = []
        for sign in (1.0, -1.0):
            sp = ac.perturbed(st, t, sign * FD_EPS)
            with ac.solver_for(sp) as g:
                vals.append(g.adjoint_forward(ac.config(nt, alpha=1.5 + sign * FD_EPS * t["alpha"])))
        fd = (vals[0] - vals[1]) / (2.0 * FD_EPS)
        mine = ac.dot(grad, t)
        worst = max(worst, abs(mine - fd) / abs(fd))
    assert worst <= TOL_FD, worst


def test_mixed_forward_and_gradient_close_to_fp64(case):
    st, nt = case
    out = {}
    for p in (abi.PRECISION_FP64, abi.PRECISION_MIXED):
        with ac.solver_for(st) as g:
            loss = g.adjoint_forward(ac.config(nt, precision=p))
            out[p] = (loss, g.adjoint_backward())
    l64, g64 = out[abi.PRECISION_FP64]
    l32, g32 = out[abi.PRECISION_MIXED]
    assert abs(l32 - l64) <= 1e-6 * abs(l64)
    for name in ("r", "v", "rho", "u"):
        scale = np.max(np.abs(g64[name]))
        assert np.max(np.abs(g32[name] - g64[name])) <= 1e-4 * scale, name
    assert abs(g32["alpha"] - g64["alpha"]) <= 1e-5 * abs(g64["alpha"])


def test_checkpoint_interval_does_not_change_result(case):
    st, nt = case
    res = []
    for k in (1, 5):
        with ac.solver_for(st) as g:
            loss = g.adjoint_forward(ac.config(nt, checkpoint=k))
            res.append((loss, g.adjoint_backward()))
    assert res[0][0] == res[1][0]
    for name in ("r", "v", "rho", "u"):
        np.testing.assert_array_equal(res[0][1][name], res[1][1][name])
    assert res[0][1]["alpha"] == res[1][1]["alpha"]


def test_partial_last_segment_and_single_list(case):
    # 13 steps: segments of 4 steps, the last one of 1; lists rebuilt every 8 steps (the second list starts
    # inside the run, not at its start)
    st, nt = case
    n = len(st["m"])
    ref, _ = oracle_loss(st, nt, steps=13, rebuild=8)
    rng = np.random.default_rng(3)
    t = ac.rough_direction(rng, n)
    _, dref = oracle_loss(st, nt, t, steps=13, rebuild=8)
    with ac.solver_for(st) as g:
        loss = g.adjoint_forward(ac.config(nt, steps=13, rebuild=8, checkpoint=4))
        grad = g.adjoint_backward()
    assert abs(loss - ref) <= 1e-13 * abs(ref)
    assert abs(ac.dot(grad, t) - dref) <= TOL_TANGENT * abs(dref)


def test_backward_repeats_and_scales(case):
    st, nt = case
    with ac.solver_for(st) as g:
        g.adjoint_forward(ac.config(nt))
        a = g.adjoint_backward(1.0)
        b = g.adjoint_backward(2.0)
    for name in ("r", "v", "rho", "u"):
        np.testing.assert_array_equal(2.0 * a[name], b[name])
    assert 2.0 * a["alpha"] == b["alpha"]


def test_no_targets_and_no_steps(case):
    st, nt = case
    with ac.solver_for(st) as g:
        assert g.adjoint_forward(ac.config(0)) == 0.0
        grad = g.adjoint_backward()
        for name in ("r", "v", "rho", "u"):
            assert not np.any(grad[name])
        loss = g.adjoint_forward(ac.config(nt, steps=0))
        v = st["v"].reshape(-1, 4)[:nt, :3]
        assert abs(loss - float(np.sum(v * v))) <= 1e-13 * loss
        grad = g.adjoint_backward()
        np.testing.assert_array_equal(grad["v"].reshape(-1, 4)[:nt, :3], 2.0 * v)
        assert not np.any(grad["r"])


def test_call_order_and_argument_errors(case):
    st, nt = case
    with ac.solver_for(st) as g:
        with pytest.raises(SphGpuError) as e:
            g.adjoint_backward()
        assert e.value.code == abi.ERR_STATE
        with pytest.raises(SphGpuError) as e:
            g.adjoint_forward(ac.config(nt, rebuild=5, checkpoint=2))
        assert e.value.code == abi.ERR_ARGUMENT
        bad = ac.config(nt)
        bad.dt = -1.0
        with pytest.raises(SphGpuError) as e:
            g.adjoint_forward(bad)
        assert e.value.code == abi.ERR_ARGUMENT
