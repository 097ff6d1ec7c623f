"""Comparison of a run with the reference's trajectory fixtures (tests/golden/*_traj_*.npz).

A trajectory fixture holds the reference's full initial state ("s0_"), its integrals, the derivatives of one
evaluation ("d0_") and, after the first step and every few steps ("t<k>_"), the state of a seeded sample of
particles ("sample_idx") together with the maximum magnitude, the sum and the sum of squares of every
component over ALL particles ("@max", "@sum", "@sum2") and the reference's integrals (TotalMomentum,
TotalAngularMomentum, TotalEnergy, each also in a frame rotating with TRAJ_FRAME_OMEGA about z).
"""
import numpy as np

# frame frequency of the "_frame" integrals of the fixtures (oracle/ref_driver.cpp, TRAJ_FRAME_OMEGA)
FRAME_OMEGA = 1.0e-4

COMPONENTS = {"r": 4, "v": 4, "dv": 4, "rho": 1, "drho": 1, "u": 1, "du": 1, "p": 1, "cs": 1, "S": 5, "dS": 5,
              "D": 1, "dD": 1}


def sampled_errors(fx, prefix, state, fields):
    """Per quantity: (max over the sampled particles of |got - ref| / max over ALL particles of |ref| (per
    component), error of the sum over all particles relative to sqrt(N * sum of squares))."""
    idx = fx["sample_idx"].astype(np.int64)
    n = len(state["m"])
    out = {}
    for f in fields:
        key = prefix + f
        if key not in fx or f not in state:
            continue
        c = COMPONENTS[f]
        got = np.asarray(state[f], dtype="f8").reshape(-1, c)
        ref = fx[key].reshape(-1, c)
        mx = fx[key + "@max"]
        err = np.max(np.abs(got[idx] - ref) / np.where(mx > 0, mx, 1.0))
        scale = np.sqrt(fx[key + "@sum2"] * n)
        esum = np.max(np.abs(got.sum(0) - fx[key + "@sum"]) / np.where(scale > 0, scale, 1.0))
        out[f] = (float(err), float(esum))
    return out


def per_particle_errors(fx, prefix, state):
    """Per-particle relative errors of quantities bounded away from zero on the sampled particles: density,
    specific energy where it exceeds 1e-3 of its maximum, smoothing length, and |v| where it exceeds 1e-2 of
    its maximum."""
    idx = fx["sample_idx"].astype(np.int64)
    out = {}
    rho = np.asarray(state["rho"])[idx]
    out["rho"] = float(np.max(np.abs(rho / fx[prefix + "rho"] - 1.0)))
    uref = fx[prefix + "u"]
    sel = np.abs(uref) > 1e-3 * fx[prefix + "u@max"][0]
    if np.any(sel):
        out["u"] = float(np.max(np.abs(np.asarray(state["u"])[idx][sel] / uref[sel] - 1.0)))
    r = np.asarray(state["r"]).reshape(-1, 4)[idx]
    rref = fx[prefix + "r"].reshape(-1, 4)
    out["h"] = float(np.max(np.abs(r[:, 3] / rref[:, 3] - 1.0)))
    v = np.linalg.norm(np.asarray(state["v"]).reshape(-1, 4)[idx, :3], axis=1)
    vref = np.linalg.norm(fx[prefix + "v"].reshape(-1, 4)[:, :3], axis=1)
    sel = vref > 1e-2 * np.max(vref) if vref.size else vref > 0
    if np.any(sel):
        out["|v|"] = float(np.max(np.abs(v[sel] / vref[sel] - 1.0)))
    return out


def integral_errors(fx, prefix, totals, totals_frame=None):
    """Errors of (momentum, angular momentum, energy) against the reference's integrals, each relative to the
    largest component of the reference's value."""
    out = {}
    p = fx[prefix + "momentum"]
    L = fx[prefix + "angular_momentum"]
    e = float(fx[prefix + "energy"][0])
    pscale = max(float(np.max(np.abs(p))), 1e-300)
    lscale = max(float(np.max(np.abs(L))), 1e-300)
    out["momentum"] = float(np.max(np.abs(totals[0:3] - p)) / pscale)
    out["angular_momentum"] = float(np.max(np.abs(totals[3:6] - L)) / lscale)
    out["energy"] = abs(float(totals[6] + totals[7]) - e) / abs(e)
    if totals_frame is not None:
        pf = fx[prefix + "momentum_frame"]
        Lf = fx[prefix + "angular_momentum_frame"]
        out["momentum_frame"] = float(np.max(np.abs(totals_frame[0:3] - pf)) / max(float(np.max(np.abs(pf))), 1e-300))
        out["angular_momentum_frame"] = float(np.max(np.abs(totals_frame[3:6] - Lf)) /
                                              max(float(np.max(np.abs(Lf))), 1e-300))
        out["energy_frame"] = abs(float(totals_frame[6] + totals_frame[7]) - float(fx[prefix + "energy_frame"][0])) / abs(e)
    return out
