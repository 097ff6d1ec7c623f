"""Shared test cases: settings and initial states rebuilt from the golden fixtures of tests/golden/.

Each fixture holds the reference's own initial state (after InitialConditions and ISolver::create), its
derivatives after one ISolver::integrate ("d0_"), the state after the first step ("s1_") and after the last
("sN_"), and the time-step sequence ("dts").
"""
import os

import numpy as np

from opensph_gb300 import abi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

STATE_FIELDS = ["r", "v", "dv", "m", "rho", "drho", "u", "du", "p", "cs", "divv", "ncnt", "flag", "corr",
                "S", "dS", "gradv", "reduce", "D", "dD", "eps_min", "m_zero", "growth", "n_flaws"]


def load(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as f:
        return {k: f[k] for k in f.files}


def kind(fx):
    """Physics of the fixture (sphere, impact, gas, ...), without the "_all" suffix of the runs with every
    time-step criterion."""
    k = str(fx["driver_args"]).split()[0]
    for suffix in ("_traj", "_cached", "_all", "_asym"):
        if k.endswith(suffix):
            k = k[:-len(suffix)]
    return k


def recomputation_period(fx):
    """gravity.recomputation_period of a run with CachedGravity (mode "<kind>_cached", last argument)."""
    args = str(fx["driver_args"]).split()
    return float(args[-1]) if args[0].endswith("_cached") else 0.0


def all_criteria(fx):
    return str(fx["driver_args"]).split()[0].endswith("_all")


def asymmetric(fx):
    """Fixture run with the AsymmetricSolver and the strain-rate correction tensor."""
    return str(fx["driver_args"]).split()[0].endswith("_asym")


def materials_of(fx):
    k = kind(fx)
    ranges = fx["mat_ranges"].reshape(-1, 6)
    mats = []
    for i, rg in enumerate(ranges):
        if k == "sphere":
            m = abi.basalt(yielding=abi.YIELDING_NONE, damage=abi.DAMAGE_NONE)
        elif k == "impact":
            m = abi.basalt()
        elif k == "gas":
            m = abi.ideal_gas(gamma=5.0 / 3.0, density=1.0)
        else:
            raise ValueError(k)
        m.density_range[:] = rg[0:2]
        m.energy_range[:] = rg[2:4]
        m.damage_range[:] = rg[4:6]
        m.young_modulus = float(fx["mat_young"][i])
        if "mat_minimals" in fx:
            m.density_min, m.energy_min, m.stress_min, m.damage_min = (float(x) for x in
                                                                       fx["mat_minimals"][4 * i:4 * i + 4])
        mats.append(m)
    return mats


def config_of(fx, precision=abi.PRECISION_FP64):
    k = kind(fx)
    n = len(fx["s0_m"])
    mats = materials_of(fx)
    crit = abi.CRITERION_ALL if all_criteria(fx) else abi.CRITERION_COURANT
    if k == "sphere":
        return abi.make_config(n, mats, forces=abi.FORCE_PRESSURE | abi.FORCE_SELF_GRAVITY,
                               gravity_constant=float(fx["G"][0]), precision=precision, timestep_criteria=crit,
                               gravity_recomputation_period=recomputation_period(fx))
    if k == "impact":
        extra = {}
        if asymmetric(fx):
            extra = {"solver_type": abi.SOLVER_ASYMMETRIC, "correction_tensor": 1}
        return abi.make_config(n, mats, forces=abi.FORCE_PRESSURE | abi.FORCE_SOLID_STRESS | abi.FORCE_SELF_GRAVITY,
                               adaptive_h=True, gravity_constant=float(fx["G"][0]), precision=precision,
                               timestep_criteria=crit, **extra)
    if k == "gas":
        return abi.make_config(n, mats, forces=abi.FORCE_PRESSURE, integrator=abi.INTEGRATOR_LEAP_FROG,
                               initial_timestep=1e-3, precision=precision, timestep_criteria=crit)
    raise ValueError(k)


def state_of(fx, prefix="s0_"):
    st = {}
    for f in STATE_FIELDS:
        key = prefix + f
        if key in fx:
            st[f] = fx[key].copy()
    st["mat"] = fx["mat"].copy()
    n = len(st["m"])
    for f in ("divv", "ncnt"):
        if f not in st:
            st[f] = np.zeros(n, dtype="u4" if f == "ncnt" else "f8")
    if "S" in st and "gradv" not in st:
        st["gradv"] = np.zeros(6 * n)
    return st


def scale_err(a, b):
    """max |a - b| / max |b| : error relative to the magnitude of the quantity over all particles."""
    a = np.asarray(a, dtype="f8")
    b = np.asarray(b, dtype="f8")
    s = np.max(np.abs(b)) if b.size else 0.0
    d = np.max(np.abs(a - b)) if b.size else 0.0
    return d / s if s > 0 else d


def vec3(a):
    return np.asarray(a).reshape(-1, 4)[:, :3]


def splitmix_uniform(seed, count):
    """The first `count` uniforms (0, 1) of the splitmix64 sequence of oracle/ref_driver.cpp (SplitMix::uniform):
    integer arithmetic and exactly rounded scaling, identical on every machine."""
    with np.errstate(over="ignore"):
        k = np.arange(1, count + 1, dtype=np.uint64)
        z = np.uint64(seed) + k * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return ((z >> np.uint64(11)).astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)


def direct_points(fx):
    """The points of a BruteForceGravity fixture (ref_driver's modeDirect): r (n x 4) and m, regenerated exactly."""
    n, seed, soft = int(fx["params"][0]), int(fx["params"][1]), float(fx["params"][2])
    u = splitmix_uniform(seed, 4 * n).reshape(n, 4)
    s = u[:, 0] * u[:, 0]
    r = np.empty((n, 4))
    for c in range(3):
        r[:, c] = s * (2.0 * u[:, c + 1] - 1.0)
    r[:, 3] = soft
    m = np.full(n, 1.0 / n)
    return r, m
