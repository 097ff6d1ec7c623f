"""ctypes mirror of include/sphgpu.h: settings structs, constants and the library loader.

The structs are the C-ABI of the GPU library; the CPU oracle under oracle/ reads the same layouts so that
both sides are driven by identical inputs.
"""
import ctypes
import os

# status codes
OK = 0
ERR_ARGUMENT = 1
ERR_ALLOCATION = 2
ERR_CAPACITY = 3
ERR_NONFINITE = 4
ERR_CUDA = 5
ERR_STATE = 6
ERR_UNSUPPORTED = 7

# quantity ids (reference QuantityId values)
Q_POSITION = 0
Q_MASS = 1
Q_PRESSURE = 2
Q_DENSITY = 3
Q_ENERGY = 4
Q_SOUND_SPEED = 5
Q_DEVIATORIC_STRESS = 6
Q_DAMAGE = 10
Q_EPS_MIN = 11
Q_M_ZERO = 12
Q_EXPLICIT_GROWTH = 13
Q_N_FLAWS = 14
Q_STRESS_REDUCING = 16
Q_ANGULAR_FREQUENCY = 20
Q_VELOCITY_GRADIENT = 26
Q_VELOCITY_DIVERGENCE = 27
Q_STRAIN_RATE_CORRECTION_TENSOR = 29
Q_NEIGHBOR_CNT = 38
Q_FLAG = 42
Q_MATERIAL_ID = 43

FORCE_PRESSURE = 1 << 0
FORCE_SOLID_STRESS = 1 << 1
FORCE_SELF_GRAVITY = 1 << 5

EOS_TILLOTSON = 0
EOS_IDEAL_GAS = 1
YIELDING_NONE = 0
YIELDING_VON_MISES = 1
DAMAGE_NONE = 0
DAMAGE_SCALAR_GRADY_KIPP = 1
INTEGRATOR_PREDICTOR_CORRECTOR = 0
INTEGRATOR_LEAP_FROG = 1
GRAVITY_KERNEL_POINT_PARTICLES = 0
GRAVITY_KERNEL_SPH_KERNEL = 1
GRAVITY_KERNEL_SOLID_SPHERES = 2
PRECISION_FP64 = 0
PRECISION_MIXED = 1

SOLVER_SYMMETRIC = 0
SOLVER_ASYMMETRIC = 1
SOLVER_NBODY_HARD_SPHERE = 2

# CollisionHandlerEnum / OverlapEnum (core/system/Settings.h:816-852)
COLLISION_NONE = 0
COLLISION_PERFECT_MERGING = 1
COLLISION_ELASTIC_BOUNCE = 2
COLLISION_MERGE_OR_BOUNCE = 3
OVERLAP_NONE = 0
OVERLAP_FORCE_MERGE = 1
OVERLAP_REPEL = 2
OVERLAP_REPEL_OR_MERGE = 3
OVERLAP_INTERNAL_BOUNCE = 4
OVERLAP_PASS_OR_MERGE = 5

CRITERION_COURANT = 1 << 1
CRITERION_DERIVATIVES = 1 << 2
CRITERION_ACCELERATION = 1 << 3
CRITERION_DIVERGENCE = 1 << 4
CRITERION_ALL = CRITERION_COURANT | CRITERION_DERIVATIVES | CRITERION_ACCELERATION | CRITERION_DIVERGENCE

# (components, numpy dtype) of each quantity across the boundary
QUANTITY_LAYOUT = {
    Q_POSITION: (4, "f8"),
    Q_MASS: (1, "f8"),
    Q_PRESSURE: (1, "f8"),
    Q_DENSITY: (1, "f8"),
    Q_ENERGY: (1, "f8"),
    Q_SOUND_SPEED: (1, "f8"),
    Q_DEVIATORIC_STRESS: (5, "f8"),
    Q_DAMAGE: (1, "f8"),
    Q_EPS_MIN: (1, "f8"),
    Q_M_ZERO: (1, "f8"),
    Q_EXPLICIT_GROWTH: (1, "f8"),
    Q_N_FLAWS: (1, "u4"),
    Q_STRESS_REDUCING: (1, "f8"),
    Q_ANGULAR_FREQUENCY: (4, "f8"),
    Q_VELOCITY_GRADIENT: (6, "f8"),
    Q_VELOCITY_DIVERGENCE: (1, "f8"),
    Q_STRAIN_RATE_CORRECTION_TENSOR: (6, "f8"),
    Q_NEIGHBOR_CNT: (1, "u4"),
    Q_FLAG: (1, "u4"),
    Q_MATERIAL_ID: (1, "u4"),
}


class Material(ctypes.Structure):
    _fields_ = [
        ("eos", ctypes.c_int32),
        ("yielding", ctypes.c_int32),
        ("damage", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("density", ctypes.c_double),
        ("bulk_modulus", ctypes.c_double),
        ("tillotson_nonlinear_b", ctypes.c_double),
        ("tillotson_small_a", ctypes.c_double),
        ("tillotson_small_b", ctypes.c_double),
        ("tillotson_alpha", ctypes.c_double),
        ("tillotson_beta", ctypes.c_double),
        ("tillotson_sublimation", ctypes.c_double),
        ("tillotson_energy_iv", ctypes.c_double),
        ("tillotson_energy_cv", ctypes.c_double),
        ("adiabatic_index", ctypes.c_double),
        ("shear_modulus", ctypes.c_double),
        ("elasticity_limit", ctypes.c_double),
        ("melt_energy", ctypes.c_double),
        ("young_modulus", ctypes.c_double),
        ("density_range", ctypes.c_double * 2),
        ("energy_range", ctypes.c_double * 2),
        ("damage_range", ctypes.c_double * 2),
        ("density_min", ctypes.c_double),
        ("energy_min", ctypes.c_double),
        ("stress_min", ctypes.c_double),
        ("damage_min", ctypes.c_double),
    ]


class Config(ctypes.Structure):
    _fields_ = [
        ("particle_count", ctypes.c_uint32),
        ("material_count", ctypes.c_uint32),
        ("materials", ctypes.POINTER(Material)),
        ("forces", ctypes.c_uint32),
        ("adaptive_smoothing_length", ctypes.c_int32),
        ("smoothing_length_range", ctypes.c_double * 2),
        ("av_alpha", ctypes.c_double),
        ("av_beta", ctypes.c_double),
        ("sum_only_undamaged", ctypes.c_int32),
        ("gravity_multipole_order", ctypes.c_int32),
        ("gravity_kernel", ctypes.c_int32),
        ("solver_type", ctypes.c_int32),
        ("gravity_constant", ctypes.c_double),
        ("gravity_opening_angle", ctypes.c_double),
        ("gravity_leaf_size", ctypes.c_uint32),
        ("integrator", ctypes.c_int32),
        ("courant_number", ctypes.c_double),
        ("max_timestep", ctypes.c_double),
        ("initial_timestep", ctypes.c_double),
        ("precision", ctypes.c_int32),
        ("device", ctypes.c_int32),
        ("timestep_criteria", ctypes.c_uint32),
        ("correction_tensor", ctypes.c_int32),
        ("derivative_factor", ctypes.c_double),
        ("divergence_factor", ctypes.c_double),
        ("max_change", ctypes.c_double),
        ("collision_handler", ctypes.c_int32),
        ("overlap_handler", ctypes.c_int32),
        ("restitution_normal", ctypes.c_double),
        ("restitution_tangent", ctypes.c_double),
        ("allowed_overlap", ctypes.c_double),
        ("bounce_merge_limit", ctypes.c_double),
        ("rotation_merge_limit", ctypes.c_double),
        ("max_bounces", ctypes.c_uint32),
        ("collision_records", ctypes.c_uint32),
        ("gravity_recomputation_period", ctypes.c_double),
    ]


INFTY = 1.7976931348623157e308
GRAVITY_CONSTANT = 6.67408e-11  # core/physics/Constants.h


def basalt(**overrides):
    """BodySettings defaults of the reference (core/system/Settings.cpp:790-960): basalt, Tillotson EOS,
    von Mises yielding and scalar Grady-Kipp damage."""
    m = Material()
    m.eos = EOS_TILLOTSON
    m.yielding = YIELDING_VON_MISES
    m.damage = DAMAGE_SCALAR_GRADY_KIPP
    m.density = 2700.0
    m.bulk_modulus = 2.67e10
    m.tillotson_nonlinear_b = 2.67e10
    m.tillotson_small_a = 0.5
    m.tillotson_small_b = 1.5
    m.tillotson_alpha = 5.0
    m.tillotson_beta = 5.0
    m.tillotson_sublimation = 4.87e8
    m.tillotson_energy_iv = 4.72e6
    m.tillotson_energy_cv = 1.82e7
    m.adiabatic_index = 1.4
    m.shear_modulus = 2.27e10
    m.elasticity_limit = 3.5e9
    m.melt_energy = 3.4e6
    m.young_modulus = 5.7e10
    m.density_range[:] = [50.0, INFTY]
    m.energy_range[:] = [0.0, INFTY]
    m.damage_range[:] = [0.0, 1.0]
    m.density_min = 100.0
    m.energy_min = 1.0
    m.stress_min = 1.0e5
    m.damage_min = 0.03
    for k, v in overrides.items():
        if k.endswith("_range"):
            getattr(m, k)[:] = v
        else:
            setattr(m, k, v)
    return m


def ideal_gas(gamma=5.0 / 3.0, density=1.0, **overrides):
    m = basalt(eos=EOS_IDEAL_GAS, yielding=YIELDING_NONE, damage=DAMAGE_NONE, adiabatic_index=gamma,
               density=density)
    for k, v in overrides.items():
        if k.endswith("_range"):
            getattr(m, k)[:] = v
        else:
            setattr(m, k, v)
    return m


def make_config(n, materials, forces=FORCE_PRESSURE | FORCE_SELF_GRAVITY, adaptive_h=False,
                integrator=INTEGRATOR_PREDICTOR_CORRECTOR, precision=PRECISION_FP64, **kw):
    """RunSettings defaults of the reference (core/system/Settings.cpp:486-730) for the fields of the path.
    Returns (config, keepalive) — keep the second value alive while the config is used."""
    arr = (Material * len(materials))(*materials)
    c = Config()
    c.particle_count = n
    c.material_count = len(materials)
    c.materials = ctypes.cast(arr, ctypes.POINTER(Material))
    c.forces = forces
    c.adaptive_smoothing_length = 1 if adaptive_h else 0
    c.smoothing_length_range[:] = [1e-5, 1e10]
    c.av_alpha = 1.5
    c.av_beta = 3.0
    c.sum_only_undamaged = 1
    c.gravity_multipole_order = 3
    c.gravity_kernel = GRAVITY_KERNEL_SPH_KERNEL
    c.gravity_constant = GRAVITY_CONSTANT
    c.gravity_opening_angle = 0.5
    c.gravity_leaf_size = 25
    c.integrator = integrator
    c.courant_number = 0.2
    c.max_timestep = 10.0
    c.initial_timestep = 0.03
    c.precision = precision
    c.device = 0
    c.timestep_criteria = CRITERION_COURANT
    c.derivative_factor = 0.2
    c.divergence_factor = 0.005
    c.max_change = INFTY
    # HardSphereSolver settings: RunSettings defaults (core/system/Settings.cpp:650-675)
    c.collision_handler = COLLISION_MERGE_OR_BOUNCE
    c.overlap_handler = OVERLAP_REPEL
    c.restitution_normal = 0.8
    c.restitution_tangent = 1.0
    c.allowed_overlap = 0.01
    c.bounce_merge_limit = 1.0
    c.rotation_merge_limit = 1.0
    c.max_bounces = 100
    for k, v in kw.items():
        if k == "smoothing_length_range":
            c.smoothing_length_range[:] = v
        else:
            setattr(c, k, v)
    return c, arr


def make_nbody_config(n, **kw):
    """The N-body run's settings (NBodyJob::getDefaultSettings, core/run/jobs/SimulationJobs.cpp:462-494):
    HardSphereSolver, leap-frog, acceleration criterion (factor 0.2), max step 10 s, initial step 0.01 s, BH
    theta 0.8 with the solid-sphere kernel and leaf size 20, MERGE_OR_BOUNCE collisions with PASS_OR_MERGE
    overlaps, restitution 0.5 / 1, merge limits 4 / 1. No materials."""
    c, keep = make_config(n, [basalt()], forces=FORCE_SELF_GRAVITY, integrator=INTEGRATOR_LEAP_FROG)
    c.material_count = 0
    c.materials = None
    c.solver_type = SOLVER_NBODY_HARD_SPHERE
    c.gravity_kernel = GRAVITY_KERNEL_SOLID_SPHERES
    c.gravity_opening_angle = 0.8
    c.gravity_leaf_size = 20
    c.timestep_criteria = CRITERION_ACCELERATION
    c.max_timestep = 10.0
    c.initial_timestep = 0.01
    c.collision_handler = COLLISION_MERGE_OR_BOUNCE
    c.overlap_handler = OVERLAP_PASS_OR_MERGE
    c.restitution_normal = 0.5
    c.restitution_tangent = 1.0
    c.allowed_overlap = 0.01
    c.bounce_merge_limit = 4.0
    c.rotation_merge_limit = 1.0
    for k, v in kw.items():
        setattr(c, k, v)
    return c, keep


class AdjointConfig(ctypes.Structure):
    """sphgpu_adjoint_config: the frozen-list hydrodynamic model differentiated by sphgpu_adjoint_*."""
    _fields_ = [
        ("steps", ctypes.c_uint32),
        ("rebuild_every", ctypes.c_uint32),
        ("checkpoint_every", ctypes.c_uint32),
        ("n_target", ctypes.c_uint32),
        ("dt", ctypes.c_double),
        ("gamma", ctypes.c_double),
        ("alpha", ctypes.c_double),
        ("beta", ctypes.c_double),
        ("precision", ctypes.c_int32),
        ("reserved", ctypes.c_uint32),
    ]


def make_adjoint_config(steps, dt, n_target, rebuild_every=10, checkpoint_every=10, gamma=5.0 / 3.0, alpha=1.5,
                        beta=3.0, precision=PRECISION_FP64):
    """StandardAV defaults alpha 1.5, beta 3 (core/system/Settings.cpp:575-578)."""
    c = AdjointConfig()
    c.steps = steps
    c.rebuild_every = rebuild_every
    c.checkpoint_every = checkpoint_every
    c.n_target = n_target
    c.dt = dt
    c.gamma = gamma
    c.alpha = alpha
    c.beta = beta
    c.precision = precision
    c.reserved = 0
    return c


_HERE = os.path.dirname(os.path.abspath(__file__))
LIBRARY_PATH = os.path.join(_HERE, "libsphgpu.so")
