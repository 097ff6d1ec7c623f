"""Inputs of the N-body (HardSphereSolver) tests: the reference fixtures tests/golden/nbody_*.npz and the
setups of the reference's own N-body tests (core/gravity/test/NBodySolver.cpp), restated here."""
import os

import numpy as np

from opensph_gb300 import abi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES = ["nbody_bounce_n1000", "nbody_merge_n1000", "nbody_default_n1000", "nbody_repel_n1000",
            "nbody_repelmerge_n1000", "nbody_internal_n1000"]
FIELDS = ["r", "v", "dv", "m", "w"]


def load(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as f:
        return {k: f[k] for k in f.files}


def config_of(fx, precision=abi.PRECISION_FP64):
    """The fixture's settings (oracle/ref_driver.cpp, modeNbody) as an N-body configuration."""
    s = fx["settings"]
    n = len(fx["s0_m"])
    return abi.make_nbody_config(
        n, collision_handler=int(s[0]), overlap_handler=int(s[1]), restitution_normal=float(s[2]),
        restitution_tangent=float(s[3]), allowed_overlap=float(s[4]), bounce_merge_limit=float(s[5]),
        rotation_merge_limit=float(s[6]), gravity_opening_angle=float(s[7]), gravity_leaf_size=int(s[8]),
        max_timestep=float(s[9]), initial_timestep=float(s[9]), derivative_factor=float(s[10]),
        gravity_constant=float(fx["G"][0]), precision=precision)


def state_of(fx, prefix):
    return {k: fx[prefix + k].copy() for k in FIELDS}


def steps_of(fx):
    return len(fx["dts"]) - 1


def scale_err(a, b):
    """max |a - b| relative to the largest magnitude of b"""
    a = np.asarray(a, dtype="f8")
    b = np.asarray(b, dtype="f8")
    if a.shape != b.shape:
        return np.inf
    s = np.abs(b).max()
    return float(np.abs(a - b).max() / s) if s > 0 else float(np.abs(a - b).max())


def kat_config(n, handler, overlap=abi.OVERLAP_NONE, dt=1.0e-4, gravity=False, **kw):
    """Settings of the reference's N-body tests: fixed step (no criterion), the handler under test."""
    return abi.make_nbody_config(
        n, collision_handler=handler, overlap_handler=overlap, timestep_criteria=0, max_timestep=dt,
        initial_timestep=dt, forces=abi.FORCE_SELF_GRAVITY if gravity else 0, **kw)


def two_particles():
    """makeTwoParticles (core/gravity/test/NBodySolver.cpp:136-147): radii 1 and 0.5 at x = +-2, mass 2,
    approaching at 10 m/s."""
    r = np.array([2.0, 0.0, 0.0, 1.0, -2.0, 0.0, 0.0, 0.5])
    v = np.array([-5.0, 0.0, 0.0, 0.0, 5.0, 0.0, 0.0, 0.0])
    return {"r": r, "v": v, "dv": np.zeros(8), "m": np.array([2.0, 2.0]), "w": np.zeros(8)}


def cloud(spacing=0.18, radius=1.0, h=0.01, k=4.0):
    """runCloud (core/gravity/test/NBodySolver.cpp:461-475): particles filling the unit sphere (here a
    cubic lattice, the reference uses its hexagonal packing), radius 0.01, velocity -4 r, so that all of
    them meet at the centre at t = 0.25."""
    g = np.arange(-radius, radius + 1e-9, spacing)
    x, y, z = np.meshgrid(g, g, g, indexing="ij")
    p = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    p = p[np.linalg.norm(p, axis=1) <= radius]
    n = len(p)
    r = np.zeros((n, 4))
    r[:, :3] = p
    r[:, 3] = h
    v = np.zeros((n, 4))
    v[:, :3] = -k * p
    m = np.full(n, 4.0 / 3.0 * np.pi / n)
    return {"r": r.ravel(), "v": v.ravel(), "dv": np.zeros(4 * n), "m": m, "w": np.zeros(4 * n)}
