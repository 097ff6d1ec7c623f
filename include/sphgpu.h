/* sphgpu.h — C ABI of the GB300 (sm_103a) implementation of OpenSPH's per-step hot path.
 *
 * One handle owns the particle state of one simulation, resident in HBM, and one CUDA stream. The entry
 * points below replace the reference's per-step C++ interfaces; the reference-side adaptor classes that
 * forward to them are in opensph_gb300/adaptor/GpuSph.h. Every function returns an sphgpu_status (0 = success); no
 * C++ exception crosses this boundary. Handles are not re-entrant: one host thread per handle at a time,
 * as the reference calls ISolver/ITimeStepping from one thread (core/timestepping/ISolver.h:22-31).
 *
 * Units and conventions follow the reference: SI units, Vector quantities are 4 doubles {x, y, z, h}
 * (core/objects/geometry/Vector.h), symmetric traceless tensors are 5 doubles {xx, yy, xy, xz, yz}
 * (core/objects/geometry/TracelessTensor.h), symmetric tensors are 6 doubles {xx, yy, zz, xy, xz, yz}
 * (core/objects/geometry/SymmetricTensor.h), index quantities are uint32 (Size).
 */
#ifndef SPHGPU_H
#define SPHGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPHGPU_ABI_VERSION 3

typedef enum {
    SPHGPU_OK = 0,
    SPHGPU_ERR_ARGUMENT = 1,    /* null pointer, size mismatch, unknown quantity, invalid setting */
    SPHGPU_ERR_ALLOCATION = 2,  /* device or pinned-host allocation failed */
    SPHGPU_ERR_CAPACITY = 3,    /* a device work list or caller buffer was too small (see sphgpu_last_error) */
    SPHGPU_ERR_NONFINITE = 4,   /* the device NaN/Inf scan found a non-finite value in the state */
    SPHGPU_ERR_CUDA = 5,        /* a CUDA runtime call failed; see sphgpu_last_error() */
    SPHGPU_ERR_STATE = 6,       /* call out of order (e.g. gravity eval before build) */
    SPHGPU_ERR_UNSUPPORTED = 7  /* a setting the GPU path does not implement */
} sphgpu_status;

/* Quantity identifiers: the numeric values of the reference's QuantityId (core/quantities/QuantityIds.h). */
enum {
    SPHGPU_Q_POSITION = 0,             /* Vector; order 0 = r, 1 = v, 2 = dv/dt */
    SPHGPU_Q_MASS = 1,                 /* double */
    SPHGPU_Q_PRESSURE = 2,             /* double */
    SPHGPU_Q_DENSITY = 3,              /* double; order 0, 1 */
    SPHGPU_Q_ENERGY = 4,               /* double; order 0, 1 */
    SPHGPU_Q_SOUND_SPEED = 5,          /* double */
    SPHGPU_Q_DEVIATORIC_STRESS = 6,    /* traceless tensor; order 0, 1 */
    SPHGPU_Q_DAMAGE = 10,              /* double; order 0, 1 */
    SPHGPU_Q_EPS_MIN = 11,             /* double */
    SPHGPU_Q_M_ZERO = 12,              /* double */
    SPHGPU_Q_EXPLICIT_GROWTH = 13,     /* double */
    SPHGPU_Q_N_FLAWS = 14,             /* uint32 */
    SPHGPU_Q_STRESS_REDUCING = 16,     /* double */
    SPHGPU_Q_ANGULAR_FREQUENCY = 20,   /* Vector {x, y, z, 0}; N-body solver only */
    SPHGPU_Q_VELOCITY_GRADIENT = 26,   /* symmetric tensor */
    SPHGPU_Q_VELOCITY_DIVERGENCE = 27, /* double */
    SPHGPU_Q_STRAIN_RATE_CORRECTION_TENSOR = 29, /* symmetric tensor (read only; with correction_tensor) */
    SPHGPU_Q_NEIGHBOR_CNT = 38,        /* uint32 */
    SPHGPU_Q_FLAG = 42,                /* uint32 */
    SPHGPU_Q_MATERIAL_ID = 43          /* uint32, index into sphgpu_config.materials */
};

/* Force flags: the reference's ForceEnum (core/system/Settings.h) bits used by this path. */
enum {
    SPHGPU_FORCE_PRESSURE = 1 << 0,
    SPHGPU_FORCE_SOLID_STRESS = 1 << 1,
    SPHGPU_FORCE_SELF_GRAVITY = 1 << 5
};

enum { SPHGPU_EOS_TILLOTSON = 0, SPHGPU_EOS_IDEAL_GAS = 1 };
enum { SPHGPU_YIELDING_NONE = 0, SPHGPU_YIELDING_VON_MISES = 1 };
enum { SPHGPU_DAMAGE_NONE = 0, SPHGPU_DAMAGE_SCALAR_GRADY_KIPP = 1 };
enum { SPHGPU_INTEGRATOR_PREDICTOR_CORRECTOR = 0, SPHGPU_INTEGRATOR_LEAP_FROG = 1 };
/* SolverEnum (core/system/Settings.h:707-729): SymmetricSolver or AsymmetricSolver. Both sum each particle's
 * neighbours in the same gather kernels here; they differ in the reference's summation order only, and the
 * asymmetric solver admits the strain-rate correction tensor. */
enum { SPHGPU_SOLVER_SYMMETRIC = 0, SPHGPU_SOLVER_ASYMMETRIC = 1 };
/* HardSphereSolver (core/gravity/NBodySolver.h:24-140): hard spheres under Barnes-Hut self-gravity with
 * collisions and overlaps resolved in time order each collide(); the state is r (radius as h), v, m and the
 * angular frequency; leap-frog only (the N-body run's integrator, core/run/jobs/SimulationJobs.cpp:467). */
enum { SPHGPU_SOLVER_NBODY_HARD_SPHERE = 2 };
/* GravityKernelEnum (core/system/Settings.h:804-814): point masses, the gravity kernel of the SPH kernel, or
 * the solid-sphere kernel of the N-body run (SolidSphereKernel, core/sph/kernel/GravityKernel.h:121-136) */
enum {
    SPHGPU_GRAVITY_KERNEL_POINT_PARTICLES = 0,
    SPHGPU_GRAVITY_KERNEL_SPH_KERNEL = 1,
    SPHGPU_GRAVITY_KERNEL_SOLID_SPHERES = 2
};
/* CollisionHandlerEnum (core/system/Settings.h:816-832, Factory::getCollisionHandler core/system/Factory.cpp:
 * 415-429): NONE ignores collisions; PERFECT_MERGING merges unconditionally; ELASTIC_BOUNCE bounces with the
 * restitution coefficients; MERGE_OR_BOUNCE merges bound pairs (escape speed and break-up spin limits) and
 * bounces the rest. */
enum {
    SPHGPU_COLLISION_NONE = 0,
    SPHGPU_COLLISION_PERFECT_MERGING = 1,
    SPHGPU_COLLISION_ELASTIC_BOUNCE = 2,
    SPHGPU_COLLISION_MERGE_OR_BOUNCE = 3
};
/* OverlapEnum (core/system/Settings.h:834-852, Factory::getOverlapHandler core/system/Factory.cpp:431-450,
 * handlers core/gravity/Collision.h:360-567). */
enum {
    SPHGPU_OVERLAP_NONE = 0,            /* overlapping pairs are ignored */
    SPHGPU_OVERLAP_FORCE_MERGE = 1,     /* merged unconditionally */
    SPHGPU_OVERLAP_REPEL = 2,           /* moved apart to touch, then bounced */
    SPHGPU_OVERLAP_REPEL_OR_MERGE = 3,  /* moved apart, then merged if bound, else bounced */
    SPHGPU_OVERLAP_INTERNAL_BOUNCE = 4, /* bounced while approaching */
    SPHGPU_OVERLAP_PASS_OR_MERGE = 5    /* merged if bound, else allowed to pass */
};
/* Time-step criteria: the reference's TimeStepCriterionEnum bits (core/system/Settings.h:577-592), evaluated
 * after every step as in MultiCriterion::compute (core/timestepping/TimeStepCriterion.cpp:139-389). */
enum {
    SPHGPU_CRITERION_COURANT = 1 << 1,      /* C h / c_s */
    SPHGPU_CRITERION_DERIVATIVES = 1 << 2,  /* f (|x| + x_min) / (|dx/dt| + EPS) of first-order quantities */
    SPHGPU_CRITERION_ACCELERATION = 1 << 3, /* f (h / |dv/dt|)^(1/2) */
    SPHGPU_CRITERION_DIVERGENCE = 1 << 4,   /* f_div / |div v| */
    SPHGPU_CRITERION_ALL = (1 << 1) | (1 << 2) | (1 << 3) | (1 << 4)
};
enum {
    SPHGPU_PRECISION_FP64 = 0, /* every operation in FP64; pair terms IEEE-identical to the reference */
    SPHGPU_PRECISION_MIXED = 1 /* FP32 cell-relative pair sums and walk, FP64 state/integrator/totals; SPH
                                  handles of fewer than 2^27 particles (the pair loop's neighbour lists hold
                                  27-bit indices; sphgpu_create refuses more with SPHGPU_ERR_UNSUPPORTED) */
};

/* One material (the reference's BodySettings entries read by EosMaterial/SolidMaterial, core/sph/Materials.cpp,
 * core/physics/Eos.cpp:198-238, core/physics/Rheology.cpp:36-83, core/physics/Damage.cpp:128-170) plus the
 * clamping ranges of IMaterial::range (core/quantities/IMaterial.h:172). */
typedef struct {
    int32_t eos;
    int32_t yielding;
    int32_t damage;
    int32_t reserved;
    double density;               /* rho0 */
    double bulk_modulus;          /* A */
    double tillotson_nonlinear_b; /* B */
    double tillotson_small_a;
    double tillotson_small_b;
    double tillotson_alpha;
    double tillotson_beta;
    double tillotson_sublimation; /* u0 */
    double tillotson_energy_iv;
    double tillotson_energy_cv;
    double adiabatic_index;       /* ideal gas gamma */
    double shear_modulus;
    double elasticity_limit;
    double melt_energy;
    double young_modulus;
    double density_range[2];
    double energy_range[2];
    double damage_range[2];
    /* IMaterial::minimal of the first-order quantities (DENSITY_MIN, ENERGY_MIN, STRESS_TENSOR_MIN, DAMAGE_MIN;
     * reference defaults 100, 1, 1e5, 0.03), used by the derivative time-step criterion */
    double density_min;
    double energy_min;
    double stress_min;
    double damage_min;
} sphgpu_material;

/* Run settings (the reference's RunSettingsId entries of the path). */
typedef struct {
    uint32_t particle_count;
    uint32_t material_count;
    const sphgpu_material* materials;
    uint32_t forces;                   /* SPHGPU_FORCE_* */
    int32_t adaptive_smoothing_length; /* AdaptiveSmoothingLength (1) or ConstSmoothingLength (0) */
    double smoothing_length_range[2];
    double av_alpha;
    double av_beta;
    int32_t sum_only_undamaged;
    int32_t gravity_multipole_order;   /* 0 (monopole), 2 (quadrupole) or 3 (octupole) */
    int32_t gravity_kernel;            /* SPHGPU_GRAVITY_KERNEL_* */
    int32_t solver_type;               /* SPHGPU_SOLVER_* */
    double gravity_constant;
    double gravity_opening_angle;
    uint32_t gravity_leaf_size;
    int32_t integrator;                /* SPHGPU_INTEGRATOR_* */
    double courant_number;
    double max_timestep;
    double initial_timestep;
    int32_t precision;                 /* SPHGPU_PRECISION_* */
    int32_t device;                    /* CUDA device ordinal */
    uint32_t timestep_criteria;        /* SPHGPU_CRITERION_* bits; 0 = Courant only */
    int32_t correction_tensor;         /* SPH_STRAIN_RATE_CORRECTION_TENSOR (CorrectionTensor, core/sph/equations/
                                        * Derivative.cpp:36-74); asymmetric solver with solid stress only */
    double derivative_factor;          /* TIMESTEPPING_DERIVATIVE_FACTOR (0.2), also the acceleration factor */
    double divergence_factor;          /* TIMESTEPPING_DIVERGENCE_FACTOR (0.005) */
    double max_change;                 /* TIMESTEPPING_MAX_INCREASE: relative growth limit of the step; 0 or
                                        * >= 1.7976931348623157e308 (the reference's INFTY, its default) = off */
    /* HardSphereSolver settings (SPHGPU_SOLVER_NBODY_HARD_SPHERE; core/system/Settings.cpp:650-675) */
    int32_t collision_handler;         /* SPHGPU_COLLISION_* (COLLISION_HANDLER) */
    int32_t overlap_handler;           /* SPHGPU_OVERLAP_* (COLLISION_OVERLAP) */
    double restitution_normal;         /* COLLISION_RESTITUTION_NORMAL */
    double restitution_tangent;        /* COLLISION_RESTITUTION_TANGENT */
    double allowed_overlap;            /* COLLISION_ALLOWED_OVERLAP */
    double bounce_merge_limit;         /* COLLISION_BOUNCE_MERGE_LIMIT */
    double rotation_merge_limit;       /* COLLISION_ROTATION_MERGE_LIMIT */
    uint32_t max_bounces;              /* COLLISION_MAX_BOUNCES */
    uint32_t collision_records;        /* collision records beyond one per particle that a collide call may create
                                        * (the work space of its time-ordered loop); 0 = max(n, 65,536) */
    /* GRAVITY_RECOMPUTATION_PERIOD (CachedGravity, core/gravity/CachedGravity.h): with a positive value the
     * self-gravity accelerations are reused while the run time is less than this period after their last
     * evaluation and the particle count is unchanged; 0 = every evaluation */
    double gravity_recomputation_period;
} sphgpu_config;

typedef struct sphgpu_handle sphgpu_handle;

/* Library / handle lifetime. */
int sphgpu_abi_version(void);
/* Replaces Factory::getSolver + ISolver::create (core/system/Factory.cpp:324, core/timestepping/ISolver.h:50):
 * validates the settings and allocates the device state for config->particle_count particles. */
sphgpu_status sphgpu_create(const sphgpu_config* config, sphgpu_handle** out);
sphgpu_status sphgpu_destroy(sphgpu_handle* h);
/* Text of the last error on this handle (or of the last failed sphgpu_create when h is NULL). */
const char* sphgpu_last_error(const sphgpu_handle* h);
/* The cudaStream_t all work of this handle is queued on (for callers that time or overlap it). */
void* sphgpu_stream(sphgpu_handle* h);
sphgpu_status sphgpu_synchronize(sphgpu_handle* h);

/* State transfer: Storage::getValue/getDt/getD2t (core/quantities/Storage.h:242) across the boundary.
 * `order` is 0 (value), 1 (first derivative) or 2 (second derivative); `count` is the particle count. */
sphgpu_status sphgpu_set_quantity(sphgpu_handle* h, int32_t id, int32_t order, const void* src, uint64_t count);
sphgpu_status sphgpu_get_quantity(sphgpu_handle* h, int32_t id, int32_t order, void* dst, uint64_t count);

/* ISymmetricFinder::build (core/objects/finders/NeighborFinder.h:101-133) on the current positions. */
sphgpu_status sphgpu_build_neighbors(sphgpu_handle* h);
/* The unordered interacting-pair set {i<j : |r_i-r_j|^2 < (2*(h_i+h_j)/2)^2} of SymmetricSolver::loop
 * (core/sph/solvers/SymmetricSolver.cpp:118-131); pairs are written as (i, j) with i < j, sorted.
 * If *npairs on return exceeds capacity, nothing beyond capacity was written (SPHGPU_ERR_CAPACITY). */
sphgpu_status sphgpu_get_pairs(sphgpu_handle* h, uint32_t* pair_i, uint32_t* pair_j, uint64_t capacity,
    uint64_t* npairs);
/* The answer of ISymmetricFinder::findAll(i, 2 h_i) (core/objects/finders/NeighborFinder.h:106-111, the query
 * radius of SymmetricSolver::loop) for every particle at once: the directed pairs (i, j), j != i, with
 * |r_j - r_i|^2 < (2 h_i)^2 (FP64), sorted by i then j; capacity semantics of sphgpu_get_pairs. */
sphgpu_status sphgpu_get_radius_pairs(sphgpu_handle* h, uint32_t* pair_i, uint32_t* pair_j, uint64_t capacity,
    uint64_t* npairs);

/* ISymmetricFinder::findAll(const Vector& pos, Float radius, Array<NeighborRecord>&)
 * (core/objects/finders/NeighborFinder.h:112-117) on the neighbour grid of the last sphgpu_build_neighbors (or
 * sphgpu_get_pairs) of the current positions: the particles j with |r_j - pos|^2 < radius^2 (x, y, z; FP64),
 * ascending in j, with those squared distances. If *count on return exceeds capacity, nothing was written
 * (SPHGPU_ERR_CAPACITY; call again with a larger capacity). SPHGPU_ERR_STATE when the positions changed since
 * the last grid build. */
sphgpu_status sphgpu_find_neighbors(sphgpu_handle* h, const double pos[3], double radius, uint32_t* indices,
    double* dist_sqr, uint64_t capacity, uint64_t* count);

/* IGravity::build + evalSelfGravity (core/gravity/IGravity.h:16-62, core/gravity/BarnesHut.cpp:50-99):
 * builds the k-d tree and multipole moments, then adds the self-gravity acceleration of every particle to
 * dv (host array of 4*count doubles, may be NULL to only update the internal acceleration buffer). The walk
 * runs in the handle's precision (FP64, or FP32 evaluation with FP64 decisions for SPHGPU_PRECISION_MIXED). */
sphgpu_status sphgpu_gravity_build(sphgpu_handle* h);
sphgpu_status sphgpu_gravity_eval(sphgpu_handle* h, double* dv, uint64_t count);
/* IGravity::evalAcceleration (core/gravity/BarnesHut.cpp:118-160) at npoints host points (4 doubles each). */
sphgpu_status sphgpu_gravity_eval_points(sphgpu_handle* h, const double* points, uint64_t npoints, double* acc);
/* IGravity::evalAttractors as BarnesHut implements it (core/gravity/BarnesHut.cpp:100-125), for the particles'
 * current positions and masses: attractors holds count x 5 doubles (position x, y, z, radius, mass). For each
 * attractor in order, every particle's dv (host, 4 doubles per particle, dv_count = particle count; may be NULL)
 * loses (G M_a) grad W(r_i - x_a, (h_i + R_a) / 2), all four components as the reference's Vector arithmetic,
 * and attractor_acc (host, 3 doubles per attractor, accumulated into) gains the sum over the particles of
 * (G m_i) grad W; then the attractor-attractor terms of each pair. At most 65,535 attractors per call. */
sphgpu_status sphgpu_gravity_attractors(sphgpu_handle* h, const double* attractors, uint64_t count,
    double* attractor_acc, double* dv, uint64_t dv_count);
/* BruteForceGravity::evalSelfGravity (core/gravity/BruteForceGravity.h:38-58, evalImpl :110-129) for the
 * particles listed in targets (host array of indices): a_i = G sum_{j != i} m_j grad W(r_j - r_i, (h_i + h_j)/2),
 * summed in FP64 over all other particles in index order; acc receives 4 doubles per target (h component 0).
 * The direct sum the Barnes-Hut walk approximates; O(targets x N). */
sphgpu_status sphgpu_gravity_direct(sphgpu_handle* h, const uint32_t* targets, uint64_t ntargets, double* acc);
/* StatisticsId::GRAVITY_NODES_APPROX / GRAVITY_NODES_EXACT / GRAVITY_NODE_COUNT of the last evaluation. */
sphgpu_status sphgpu_gravity_stats(sphgpu_handle* h, uint64_t out[3]);
/* Interactions evaluated by the last walk: out[0] particle-multipole evaluations (sum over leaves of
 * particles x node-list length), out[1] particle-particle kernel evaluations (particle lists and pairs
 * inside each leaf). */
sphgpu_status sphgpu_gravity_interactions(sphgpu_handle* h, uint64_t out[2]);

/* ISolver::integrate (core/sph/solvers/SymmetricSolver.cpp:58-95 wrapped by GravitySolver::loop,
 * core/sph/solvers/GravitySolver.cpp:64-91): materials initialize, gravity, pair loop, finalize. The
 * highest derivatives are overwritten (the caller's zeroHighestDerivatives is implied). With the N-body solver
 * HardSphereSolver::integrate (core/gravity/NBodySolver.cpp:97-117): dv = self-gravity, h derivatives 0. */
sphgpu_status sphgpu_integrate(sphgpu_handle* h);

/* ITimeStepping::step x nsteps (core/timestepping/TimeStepping.cpp:34-75, PredictorCorrector :272-346,
 * LeapFrog :352-391) followed each step by the time-step criteria (core/timestepping/TimeStepCriterion.cpp:
 * 139-389). Runs asynchronously on the handle's stream; the time step stays on the device. With the N-body
 * solver each leap-frog step is collide(dt/2), drift, integrate, kick, collide(dt/2), drift (the collisions
 * synchronise the stream twice per step). */
sphgpu_status sphgpu_step(sphgpu_handle* h, uint32_t nsteps);
sphgpu_status sphgpu_get_timestep(sphgpu_handle* h, double* dt);
sphgpu_status sphgpu_set_timestep(sphgpu_handle* h, double dt);
/* Run time (StatisticsId::RUN_TIME): 0 at creation, advanced by every step by the step taken. */
sphgpu_status sphgpu_get_time(sphgpu_handle* h, double* t);
sphgpu_status sphgpu_set_time(sphgpu_handle* h, double t);

/* HardSphereSolver::collide (core/gravity/NBodySolver.cpp:329-484) over the interval [0, dt): finds every
 * particle's earliest collision or overlap, resolves them in time order (re-searching the particles whose
 * pending collisions were invalidated), and removes merged particles, keeping the order of the others
 * (Storage::remove). N-body solver only; sphgpu_step calls it twice per leap-frog step. When the collision
 * work space (pool_capacity records) runs out, SPHGPU_ERR_CAPACITY is returned with the collisions processed
 * until then applied and their merged particles removed (mass and momentum conserved); the interval's remaining
 * collisions are not processed. */
sphgpu_status sphgpu_collide(sphgpu_handle* h, double dt);
/* Current particle count (changes when collisions merge particles). */
sphgpu_status sphgpu_particle_count(sphgpu_handle* h, uint64_t* n);
/* The indices, ascending and in the numbering of the last call of this function (or of the last position
 * upload), of the particles removed by merging since then; the numbering restarts from the current state. The
 * argument of the reference's Storage::remove (core/quantities/Storage.h) for a host copy of the state. If
 * more than `capacity` were removed, *count says how many and SPHGPU_ERR_CAPACITY is returned (call again). */
sphgpu_status sphgpu_take_removed(sphgpu_handle* h, uint32_t* removed, uint64_t capacity, uint64_t* count);
/* StatisticsId::TOTAL_COLLISION_COUNT, MERGER_COUNT, BOUNCE_COUNT, OVERLAP_COUNT (core/gravity/NBodySolver.cpp:
 * 119-163), summed over all collide calls since the handle was created. */
sphgpu_status sphgpu_collision_stats(sphgpu_handle* h, uint64_t out[4]);
/* Profile of the collision loop summed over all collide calls: out[0] records processed, out[1..3] SM clock
 * cycles spent in its serial part (selection, handler, invalidation), in the re-searches and in inserting the
 * new records. */
sphgpu_status sphgpu_collision_profile(sphgpu_handle* h, uint64_t out[4]);

/* Conserved totals (core/physics/Integrals.h:62-148) as compensated FP64 device reductions:
 * out[0..2] momentum, out[3..5] angular momentum about the origin, out[6] kinetic energy,
 * out[7] internal energy, out[8] total mass. */
sphgpu_status sphgpu_totals(sphgpu_handle* h, double out[9]);
/* The same totals in a frame rotating with frequency omega about z: TotalMomentum(omega) and
 * TotalAngularMomentum(omega) (core/physics/Integrals.cpp:20-62) use v + omega x r; the kinetic energy uses v,
 * as TotalEnergy(omega) does (Integrals.cpp:64-91). sphgpu_totals is omega = 0. */
sphgpu_status sphgpu_totals_frame(sphgpu_handle* h, double omega, double out[9]);

/* Device NaN/Inf scan of the integrated state; SPHGPU_ERR_NONFINITE with the first bad particle index. */
sphgpu_status sphgpu_check_finite(sphgpu_handle* h, uint64_t* first_bad);

/* Measured FP32 FMA rate of the current device in TFLOP/s (independent FMA chains on every SM, one launch of about
 * ms_target milliseconds timed with CUDA events): the denominator of FP32 roofline reports. No counterpart in the
 * reference. */
sphgpu_status sphgpu_measure_fp32_peak(double ms_target, double* tflops);

/* Conserved totals without any allocation (no counterpart in the reference). For callers that cannot call
 * cudaMalloc: an application that owns the device memory budget and passes only its own buffers, or a
 * per-step hook that must not risk the implicit synchronisation of an allocation. r, v (4 doubles per
 * particle), m, u (1 double per particle) and totals (9 doubles, layout of sphgpu_totals) are DEVICE
 * pointers of the current device; the work is queued on `stream` (a cudaStream_t, NULL for the default
 * stream) and the call returns without synchronising. The scratch is a fixed 72 KiB array inside the
 * library, shared by all calls: calls whose kernels overlap on the GPU race, so serialise them. Each call
 * looks up that array's device address for the current device (a host-side query); the first call on a device
 * may load the library's device code, so make it before any stream capture.
 * n above SPHGPU_TOTALS_NOALLOC_MAX_PARTICLES returns SPHGPU_ERR_CAPACITY (use sphgpu_totals). */
#define SPHGPU_TOTALS_NOALLOC_MAX_PARTICLES 4194304u
sphgpu_status sphgpu_totals_noalloc(const double* r, const double* v, const double* m, const double* u, uint64_t n,
    double* totals, void* stream);

/* Adjoint of the frozen-list hydrodynamic step (no counterpart in the reference, which has no
 * differentiation). The model: ideal gas p = (gamma - 1) u rho (IdealGasEos, core/physics/Eos.cpp:42-45),
 * ContinuityEquation + PressureForce + StandardAV (core/sph/equations/EquationTerm.cpp:42-99, 289-316,
 * core/sph/equations/av/Standard.h:63-83) with the cubic-spline LUT kernel, leap-frog
 * (core/timestepping/TimeStepping.cpp:352-391) with the fixed step dt and constant h. The neighbour lists
 * (|r_i - r_j| < 2 * 0.5 (h_i + h_j)) are rebuilt every rebuild_every steps and held fixed in between.
 * Loss = sum over particles [0, n_target) of |v|^2 after `steps` steps.
 * sphgpu_adjoint_forward runs the model from the handle's r, v, m, rho, u (left unchanged) and returns the
 * loss; it keeps a checkpoint every checkpoint_every steps in device memory (checkpoint_every must divide
 * rebuild_every). sphgpu_adjoint_backward then returns loss_bar times the gradient of the loss with respect
 * to the initial r and v (4 doubles per particle, the 4th = 0: h is not differentiated), rho, u and the AV
 * alpha, recomputing each segment between checkpoints; outputs are host buffers, any may be NULL. Both use
 * the handle's neighbour grid (call sphgpu_build_neighbors again before sphgpu_get_pairs). precision:
 * SPHGPU_PRECISION_FP64 or SPHGPU_PRECISION_MIXED (FP32 pair terms, FP64 state and update). */
typedef struct {
    uint32_t steps;
    uint32_t rebuild_every;
    uint32_t checkpoint_every;
    uint32_t n_target;
    double dt;
    double gamma;   /* adiabatic index */
    double alpha;   /* StandardAV alpha (differentiated) */
    double beta;    /* StandardAV beta */
    int32_t precision;
    uint32_t reserved;
} sphgpu_adjoint_config;
sphgpu_status sphgpu_adjoint_forward(sphgpu_handle* h, const sphgpu_adjoint_config* cfg, double* loss);
sphgpu_status sphgpu_adjoint_backward(sphgpu_handle* h, double loss_bar, double* grad_r, double* grad_v,
    double* grad_rho, double* grad_u, double* grad_alpha);

/* Phases of a step, timed with CUDA events when profiling is on; the GPU counterparts of the reference's
 * StatisticsId::GRAVITY_BUILD_TIME, GRAVITY_EVAL_TIME and SPH_EVAL_TIME (core/system/Statistics.h:108-160,
 * set at core/sph/solvers/GravitySolver.cpp:71-90). */
enum {
    SPHGPU_PHASE_PREDICT = 0,       /* predictor (or leap-frog drift) + EOS / rheology initialize */
    SPHGPU_PHASE_GRAVITY_BUILD = 1, /* k-d tree + multipole moments */
    SPHGPU_PHASE_GRAVITY_EVAL = 2,  /* tree walk */
    SPHGPU_PHASE_NEIGHBORS = 3,     /* neighbour grid build + cell-sorted copies */
    SPHGPU_PHASE_SPH_EVAL = 4,      /* pair loop + finalize + fracture model */
    SPHGPU_PHASE_CORRECT = 5,       /* corrector (or leap-frog kick) + Courant criterion */
    SPHGPU_PHASE_COLLIDE = 6,       /* N-body collision search and resolution (COLLISION_EVAL_TIME) */
    SPHGPU_PHASE_WALK_EVALUATION = 7, /* the tree walk's evaluation kernel alone (inside GRAVITY_EVAL, which also
                                         holds the walk's interaction-list phase) */
    SPHGPU_PHASE_COUNT = 8
};
sphgpu_status sphgpu_set_profiling(sphgpu_handle* h, int32_t enabled);
/* Device milliseconds per phase and the number of this library's kernel launches since the last call
 * (synchronizes the stream; resets the accumulators). Either output may be NULL. */
sphgpu_status sphgpu_phase_times(sphgpu_handle* h, double out[SPHGPU_PHASE_COUNT], uint64_t* launches);

#ifdef __cplusplus
}
#endif

#endif /* SPHGPU_H */
