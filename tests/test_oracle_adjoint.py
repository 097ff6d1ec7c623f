"""The oracle's FP64 tangent-linear model of the frozen-list hydrodynamic step (the reference for the GPU
adjoint) against its own central finite differences, in 8 seeded smooth directions; and the kink that the
contracting initial state avoids."""
import numpy as np

import adjoint_cases as ac
from oracle import oracle


def _loss(st, nt, t=None, alpha=1.5):
    return oracle.frozen_loss(st["r"], st["v"], st["m"], st["rho"], st["u"], ac.STEPS, ac.DT, nt,
                              rebuild_every=ac.REBUILD, alpha=alpha, tangent=t)


def test_tangent_linear_matches_central_differences():
    st, nt = ac.gas_state()
    rng = np.random.default_rng(5)
    eps = 1e-6
    for _ in range(8):
        t = ac.smooth_direction(rng, st, nt)
        _, d = _loss(st, nt, t)
        lp, _ = _loss(ac.perturbed(st, t, eps), nt, alpha=1.5 + eps * t["alpha"])
        lm, _ = _loss(ac.perturbed(st, t, -eps), nt, alpha=1.5 - eps * t["alpha"])
        fd = (lp - lm) / (2.0 * eps)
        assert abs(d - fd) <= 1e-5 * abs(fd), (d, fd)


def test_tangent_is_linear():
    st, nt = ac.gas_state()
    n = len(st["m"])
    rng = np.random.default_rng(8)
    a, b = ac.rough_direction(rng, n), ac.rough_direction(rng, n)
    combo = {k: (2.0 * a[k] - 0.5 * b[k]) for k in a}
    _, da = _loss(st, nt, a)
    _, db = _loss(st, nt, b)
    _, dc = _loss(st, nt, combo)
    assert abs(dc - (2.0 * da - 0.5 * db)) <= 1e-10 * (abs(2.0 * da) + abs(0.5 * db))


def test_bodies_at_rest_sit_on_the_viscosity_switch():
    # with no contraction every pair inside a body has v_ij . r_ij = 0 at the start, where the AV term has a
    # kink: a velocity finite difference then disagrees with the one-sided tangent at the 1e-3 level
    st, nt = ac.gas_state(compression=0.0)
    n = len(st["m"])
    rng = np.random.default_rng(2)
    tv = rng.standard_normal((n, 4))
    tv[:, 3] = 0.0
    t = {"v": tv.ravel()}
    _, d = _loss(st, nt, t)
    eps = 1e-6
    lp, _ = _loss(ac.perturbed(st, t, eps), nt)
    lm, _ = _loss(ac.perturbed(st, t, -eps), nt)
    fd = (lp - lm) / (2.0 * eps)
    assert abs(d - fd) > 1e-4 * abs(fd)
