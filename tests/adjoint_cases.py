"""Shared set-up of the adjoint tests: the gas-impact state, seeded directions and the FP64 directional
derivative of the frozen-list loss from the oracle's tangent-linear model."""
import numpy as np

from opensph_gb300 import abi, initial
from opensph_gb300.solver import GpuSolver

STEPS = 20
DT = 2.0e-3
REBUILD = 5
CHECKPOINT = 5


def gas_state(n_target=2000, n_imp=100, **kw):
    st, nt = initial.gas_impact(n_target, n_imp, **kw)
    return st, nt


def solver_for(st):
    n = len(st["m"])
    cfg, keep = abi.make_config(n, [abi.ideal_gas()], forces=abi.FORCE_PRESSURE)
    g = GpuSolver(cfg, keep)
    g.set_state({"r": st["r"], "v": st["v"], "m": st["m"], "rho": st["rho"], "u": st["u"]})
    return g


def config(nt, steps=STEPS, rebuild=REBUILD, checkpoint=CHECKPOINT, precision=abi.PRECISION_FP64, alpha=1.5):
    return abi.make_adjoint_config(steps, DT, nt, rebuild_every=rebuild, checkpoint_every=checkpoint,
                                   alpha=alpha, precision=precision)


def rough_direction(rng, n):
    """Independent normal perturbations of every r, v, rho, u component and of alpha (h not perturbed)."""
    t = {}
    for name, comps in (("r", 4), ("v", 4), ("rho", 1), ("u", 1)):
        a = rng.standard_normal((n, comps))
        if comps == 4:
            a[:, 3] = 0.0
        t[name] = a.ravel()
    t["rho"] *= 1e-2
    t["u"] *= 1e-2
    t["alpha"] = float(rng.standard_normal())
    return t


def smooth_direction(rng, st, nt):
    """A smooth displacement field of all positions (three random Fourier modes), a common velocity change of
    the impactor and a change of alpha. Smooth fields keep a finite difference clear of the kinks of the model
    (nodes of the kernel table, the AV switch, neighbour-list membership), which per-particle noise crosses."""
    n = len(st["m"])
    pos = st["r"].reshape(-1, 4)[:, :3]
    dr = np.zeros((n, 4))
    for _ in range(3):
        k = 2.0 * rng.standard_normal(3)
        phase = 2.0 * np.pi * rng.random()
        amp = rng.standard_normal(3)
        dr[:, :3] += np.sin(pos @ k + phase)[:, None] * amp[None, :]
    dv = np.zeros((n, 4))
    dv[nt:, :3] = rng.standard_normal(3)
    return {"r": dr.ravel(), "v": dv.ravel(), "alpha": float(rng.standard_normal())}


def dot(grad, t):
    out = 0.0
    for name in ("r", "v", "rho", "u"):
        if name in t:
            out += float(np.dot(grad[name], t[name]))
    return out + grad["alpha"] * t.get("alpha", 0.0)


def perturbed(st, t, eps):
    out = {k: v.copy() for k, v in st.items()}
    for name in ("r", "v", "rho", "u"):
        if name in t:
            out[name] = out[name] + eps * t[name]
    return out
