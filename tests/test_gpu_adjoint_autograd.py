"""Gradient harness: the C ABI pair sphgpu_adjoint_forward / sphgpu_adjoint_backward wrapped in a thin
torch.autograd.Function (test-only; the library itself has no torch dependency).

torch.autograd.grad through the wrapper must return exactly the gradients of a direct backward call, and a
directional derivative assembled from them must match the oracle's FP64 tangent-linear run and an FP64 central
finite difference computed through the same wrapper.
"""
import numpy as np
import pytest

import adjoint_cases as ac
from oracle import oracle

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


class FrozenLoss(torch.autograd.Function):
    """loss = sum over targets |v(T)|^2 of the frozen-list model from (r, v, alpha); rho, u, m held fixed."""

    @staticmethod
    def forward(ctx, r, v, alpha, base, nt, precision):
        st = dict(base)
        st["r"] = r.detach().cpu().numpy().astype("f8")
        st["v"] = v.detach().cpu().numpy().astype("f8")
        g = ac.solver_for(st)
        loss = g.adjoint_forward(ac.config(nt, precision=precision, alpha=float(alpha)))
        ctx.solver = g
        return torch.tensor(loss, dtype=torch.float64)

    @staticmethod
    def backward(ctx, loss_bar):
        g = ctx.solver
        grad = g.adjoint_backward(float(loss_bar))
        g.close()
        ctx.solver = None
        return (torch.from_numpy(grad["r"]), torch.from_numpy(grad["v"]),
                torch.tensor(grad["alpha"], dtype=torch.float64), None, None, None)


def test_autograd_wrapper_matches_abi_and_references():
    st, nt = ac.gas_state()
    n = len(st["m"])
    r = torch.tensor(st["r"], dtype=torch.float64, requires_grad=True)
    v = torch.tensor(st["v"], dtype=torch.float64, requires_grad=True)
    alpha = torch.tensor(1.5, dtype=torch.float64, requires_grad=True)
    loss = FrozenLoss.apply(r, v, alpha, st, nt, 0)
    gr, gv, ga = torch.autograd.grad(3.0 * loss, [r, v, alpha])

    with ac.solver_for(st) as g:
        direct_loss = g.adjoint_forward(ac.config(nt))
        direct = g.adjoint_backward(3.0)
    assert float(loss.detach()) == direct_loss
    np.testing.assert_array_equal(gr.numpy(), direct["r"])
    np.testing.assert_array_equal(gv.numpy(), direct["v"])
    assert float(ga) == direct["alpha"]

    rng = np.random.default_rng(21)
    t = ac.rough_direction(rng, n)
    del t["rho"], t["u"]
    _, ref = oracle.frozen_loss(st["r"], st["v"], st["m"], st["rho"], st["u"], ac.STEPS, ac.DT, nt,
                                rebuild_every=ac.REBUILD, tangent=t)
    mine = (float(torch.dot(gr, torch.from_numpy(t["r"]))) + float(torch.dot(gv, torch.from_numpy(t["v"])))
            + float(ga) * t["alpha"]) / 3.0
    assert abs(mine - ref) <= 1e-9 * abs(ref)

    # central difference through the wrapper along a smooth direction
    t = ac.smooth_direction(rng, st, nt)
    eps = 1e-6
    with torch.no_grad():
        lp = FrozenLoss.apply(r + eps * torch.from_numpy(t["r"]), v + eps * torch.from_numpy(t["v"]),
                              alpha + eps * t["alpha"], st, nt, 0)
        lm = FrozenLoss.apply(r - eps * torch.from_numpy(t["r"]), v - eps * torch.from_numpy(t["v"]),
                              alpha - eps * t["alpha"], st, nt, 0)
    fd = float(lp - lm) / (2.0 * eps)
    mine = (float(torch.dot(gr, torch.from_numpy(t["r"]))) + float(torch.dot(gv, torch.from_numpy(t["v"])))
            + float(ga) * t["alpha"]) / 3.0
    assert abs(mine - fd) <= 1e-4 * abs(fd)
