// abi.cu — the C ABI of libsphgpu (include/sphgpu.h): handle lifetime, state transfer and the per-step
// orchestration of the kernels (the GB300 replacement of ITimeStepping::step -> ISolver::integrate ->
// GravitySolver::loop -> SymmetricSolver::loop, core/timestepping/TimeStepping.cpp:34-391,
// core/sph/solvers/GravitySolver.cpp:64-91, core/sph/solvers/SymmetricSolver.cpp:58-141).

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "state.h"

using namespace sphgpu;

struct sphgpu_handle {
    sphgpu_config cfg;
    std::vector<sphgpu_material> materials;
    Physics ph;
    DState s;
    Grid grid;
    Tree tree;
    MaterialD* d_mats = nullptr;
    double* d_lut_sph = nullptr;   // LutKernel<3>(CubicSpline<3>) gradient table
    double* d_lut_grav = nullptr;  // LutKernel<3>(GravityKernel<CubicSpline<3>>) gradient table
    float* d_lut_sph_f = nullptr;
    float* d_lut_grav_f = nullptr;
    double* d_dt = nullptr;
    double* d_dt_min = nullptr;
    double* d_time = nullptr;      // run time (StatisticsId::RUN_TIME), advanced by every step
    // CachedGravity (core/gravity/CachedGravity.h): time and particle count of the last gravity evaluation,
    // and whether the current evaluation reuses it
    double gravity_t_last = -INFINITY;
    uint32_t gravity_n_last = 0;
    bool gravity_cached = false;
    uint32_t* d_err = nullptr;
    double* d_tot_partial = nullptr;
    double* d_tot = nullptr;
    unsigned long long* d_count = nullptr;
    unsigned long long* h_pinned = nullptr; // small pinned scratch for device->host scalars
    cudaStream_t stream = nullptr;
    std::vector<void*> allocations;
    std::string error;
    bool gravity_current = false;
    // the neighbour grid of sphgpu_build_neighbors is that of the current positions (point queries use it)
    bool grid_current = false;
    // profiling: device time per phase (CUDA events on the handle's stream) and own kernel launches
    bool profiling = false;
    std::vector<cudaEvent_t> event_pool;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> marks;
    double phase_ms[SPHGPU_PHASE_COUNT] = { 0 };
    unsigned long long launches = 0;
    // adjoint of the frozen-list hydrodynamic step (allocated by the first sphgpu_adjoint_forward)
    AdjointState* adjoint = nullptr;
    // self-gravity runs on its own higher-priority stream, concurrently with the SPH pair loop
    cudaStream_t gstream = nullptr;
    cudaEvent_t ev_fork = nullptr;
    cudaEvent_t ev_join = nullptr;
    // HardSphereSolver: collision work space and settings, and the interval of sphgpu_collide
    Collide coll;
    CollideParams cp;
    double* d_dtc = nullptr;
    uint32_t n_sync = 0; // particle count at the last sphgpu_take_removed / position upload
};

namespace {

thread_local std::string gCreateError;

sphgpu_status fail(sphgpu_handle* h, sphgpu_status code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (h) {
        h->error = buf;
    } else {
        gCreateError = buf;
    }
    return code;
}

sphgpu_status cudaFail(sphgpu_handle* h, cudaError_t e, const char* where) {
    return fail(h, SPHGPU_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
}

cudaEvent_t takeEvent(sphgpu_handle* h) {
    if (!h->event_pool.empty()) {
        cudaEvent_t e = h->event_pool.back();
        h->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Scoped phase timer: records a start/end event pair on the stream when profiling is on.
struct Phase {
    sphgpu_handle* h;
    int id;
    cudaStream_t stream;
    cudaEvent_t start = nullptr;
    Phase(sphgpu_handle* hh, int phase) : Phase(hh, phase, hh->stream) {}
    Phase(sphgpu_handle* hh, int phase, cudaStream_t st) : h(hh), id(phase), stream(st) {
        if (h->profiling) {
            start = takeEvent(h);
            cudaEventRecord(start, stream);
        }
    }
    ~Phase() {
        if (h->profiling && start) {
            cudaEvent_t end = takeEvent(h);
            cudaEventRecord(end, stream);
            h->marks.push_back({ id, { start, end } });
        }
    }
};

#define CUDA_TRY(h, call)                                                                                        \
    do {                                                                                                         \
        cudaError_t e_ = (call);                                                                                 \
        if (e_ != cudaSuccess) {                                                                                 \
            return cudaFail(h, e_, #call);                                                                       \
        }                                                                                                        \
    } while (0)

// ---- LUT tables: the reference's LutKernel construction (core/sph/kernel/Kernel.h:51-100) ----------------

const double kPi = 3.14159265358979323846264338327950288419716939937510;

double cubicGrad(double qSqr) {
    const double norm = 1. / kPi;
    const double q = std::sqrt(qSqr);
    if (q == 0.) {
        return -3. * norm;
    }
    if (q < 1.) {
        const double a = 2. - q, b = 1. - q;
        return (1. / q) * norm * (-0.75 * (a * a) + 3. * (b * b));
    }
    if (q < 2.) {
        const double a = 2. - q;
        return (1. / q) * norm * (-0.75 * (a * a));
    }
    return 0.;
}

double gravGrad(double qSqr) {
    const double q = std::sqrt(qSqr);
    if (q == 0.) {
        return 4. / 3.;
    }
    if (q < 1.) {
        return 1. / q * (4. / 3. * q - 6. / 5. * (q * q * q) + 1. / 2. * (qSqr * qSqr));
    }
    return 1. / q *
           (8. / 3. * q - 3. * qSqr + 6. / 5. * (q * q * q) - 1. / 6. * (qSqr * qSqr) - 1. / (15. * qSqr));
}

template <typename F>
std::vector<double> makeLut(F f) {
    const double rad = 2.;
    const double radInvSqr = 1. / (rad * rad);
    const double qSqrToIdx = double(LUT_ENTRIES) * radInvSqr;
    std::vector<double> out(LUT_ENTRIES + 1);
    for (int i = 0; i < LUT_ENTRIES + 1; ++i) {
        out[i] = f(double(i) / qSqrToIdx);
    }
    return out;
}

MaterialD toDevice(const sphgpu_material& m) {
    MaterialD d;
    d.eos = m.eos;
    d.yielding = m.yielding;
    d.damage = m.damage;
    d.pad = 0;
    d.rho0 = m.density;
    d.A = m.bulk_modulus;
    d.B = m.tillotson_nonlinear_b;
    d.a = m.tillotson_small_a;
    d.b = m.tillotson_small_b;
    d.alpha = m.tillotson_alpha;
    d.beta = m.tillotson_beta;
    d.u0 = m.tillotson_sublimation;
    d.uiv = m.tillotson_energy_iv;
    d.ucv = m.tillotson_energy_cv;
    d.gamma = m.adiabatic_index;
    d.mu = m.shear_modulus;
    d.limit = m.elasticity_limit;
    d.u_melt = m.melt_energy;
    d.young = m.young_modulus;
    d.rho_lo = m.density_range[0];
    d.rho_hi = m.density_range[1];
    d.u_lo = m.energy_range[0];
    d.u_hi = m.energy_range[1];
    d.d_lo = m.damage_range[0];
    d.d_hi = m.damage_range[1];
    d.rho_min = m.density_min;
    d.u_min = m.energy_min;
    d.s_min = m.stress_min;
    d.d_min = m.damage_min;
    d.inv_rho0 = d.rho0 != 0. ? 1. / d.rho0 : 0.;
    d.inv_u0 = d.u0 != 0. ? 1. / d.u0 : 0.;
    d.inv_u_melt = d.u_melt != 0. ? 1. / d.u_melt : 0.;
    return d;
}

template <typename T>
cudaError_t devAlloc(sphgpu_handle* h, T** p, size_t count) {
    void* ptr = nullptr;
    cudaError_t e = cudaMalloc(&ptr, std::max<size_t>(count * sizeof(T), 16));
    if (e == cudaSuccess) {
        cudaMemset(ptr, 0, std::max<size_t>(count * sizeof(T), 16));
        h->allocations.push_back(ptr);
        *p = static_cast<T*>(ptr);
    }
    return e;
}

struct QuantitySlot {
    void* dev;     // device base pointer
    int comps;     // components per particle
    int bytes;     // bytes per component
    bool soa;      // component-major on the device
};

// Maps (quantity, order) to the device buffer; dev == nullptr if the handle does not hold it.
bool slotOf(sphgpu_handle* h, int id, int order, QuantitySlot& q) {
    DState& s = h->s;
    q = QuantitySlot{ nullptr, 1, 8, false };
    switch (id) {
    case SPHGPU_Q_POSITION:
        q.comps = 4;
        q.dev = order == 0 ? (void*)s.r : (order == 1 ? (void*)s.v : (order == 2 ? (void*)s.dv : nullptr));
        return order >= 0 && order <= 2;
    case SPHGPU_Q_MASS:
        q.dev = s.m;
        return order == 0;
    case SPHGPU_Q_PRESSURE:
        q.dev = s.p;
        return order == 0;
    case SPHGPU_Q_DENSITY:
        q.dev = order == 0 ? (void*)s.rho : (void*)s.drho;
        return order == 0 || order == 1;
    case SPHGPU_Q_ENERGY:
        q.dev = order == 0 ? (void*)s.u : (void*)s.du;
        return order == 0 || order == 1;
    case SPHGPU_Q_SOUND_SPEED:
        q.dev = s.cs;
        return order == 0;
    case SPHGPU_Q_DEVIATORIC_STRESS:
        q.comps = 5;
        q.soa = true;
        q.dev = order == 0 ? (void*)s.S : (void*)s.dS;
        return order == 0 || order == 1;
    case SPHGPU_Q_DAMAGE:
        q.dev = order == 0 ? (void*)s.D : (void*)s.dD;
        return order == 0 || order == 1;
    case SPHGPU_Q_EPS_MIN:
        q.dev = s.eps_min;
        return order == 0;
    case SPHGPU_Q_M_ZERO:
        q.dev = s.m_zero;
        return order == 0;
    case SPHGPU_Q_EXPLICIT_GROWTH:
        q.dev = s.growth;
        return order == 0;
    case SPHGPU_Q_N_FLAWS:
        q.bytes = 4;
        q.dev = s.n_flaws;
        return order == 0;
    case SPHGPU_Q_STRESS_REDUCING:
        q.dev = s.reduce;
        return order == 0;
    case SPHGPU_Q_ANGULAR_FREQUENCY:
        q.comps = 4;
        q.dev = s.omega;
        return order == 0;
    case SPHGPU_Q_VELOCITY_GRADIENT:
        q.comps = 6;
        q.soa = true;
        q.dev = s.gradv;
        return order == 0;
    case SPHGPU_Q_VELOCITY_DIVERGENCE:
        q.dev = s.divv;
        return order == 0;
    case SPHGPU_Q_STRAIN_RATE_CORRECTION_TENSOR:
        q.comps = 6;
        q.soa = true;
        q.dev = s.corr;
        return order == 0;
    case SPHGPU_Q_NEIGHBOR_CNT:
        q.bytes = 4;
        q.dev = s.ncnt;
        return order == 0;
    case SPHGPU_Q_FLAG:
        q.bytes = 4;
        q.dev = s.flag;
        return order == 0;
    case SPHGPU_Q_MATERIAL_ID:
        q.bytes = 4;
        q.dev = s.mat;
        return order == 0;
    default:
        return false;
    }
}

sphgpu_status checkDeviceError(sphgpu_handle* h) {
    cudaError_t e = cudaMemcpyAsync(h->h_pinned, h->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) {
        e = cudaStreamSynchronize(h->stream);
    }
    if (e != cudaSuccess) {
        return cudaFail(h, e, "device error check");
    }
    const uint32_t err = *reinterpret_cast<uint32_t*>(h->h_pinned);
    if (err) {
        cudaMemsetAsync(h->d_err, 0, sizeof(uint32_t), h->stream);
        cudaStreamSynchronize(h->stream);
        return fail(h, SPHGPU_ERR_CAPACITY, "device work list overflow (error bits 0x%x)", err);
    }
    return SPHGPU_OK;
}

// gravity build + walk into s.agrav (GravitySolver::loop, first half)
// BarnesHut::build + evalSelfGravity into s.agrav, queued on stream st
sphgpu_status evalGravityBuild(sphgpu_handle* h, cudaStream_t st) {
    if (h->gravity_cached) {
        return SPHGPU_OK; // CachedGravity: s.agrav still holds the accelerations of the last evaluation
    }
    Phase ph(h, SPHGPU_PHASE_GRAVITY_BUILD, st);
    cudaError_t e = treeBuild(h->s, h->tree, h->ph, h->d_err, st);
    if (e != cudaSuccess) {
        return cudaFail(h, e, "gravity build");
    }
    h->launches += h->tree.launches;
    return SPHGPU_OK;
}

sphgpu_status evalGravityWalk(sphgpu_handle* h, cudaStream_t st) {
    if (h->gravity_cached) {
        return SPHGPU_OK;
    }
    {
        Phase ph(h, SPHGPU_PHASE_GRAVITY_EVAL, st);
        // the evaluation kernel alone, timed inside the phase
        cudaEvent_t e0 = h->profiling ? takeEvent(h) : nullptr, e1 = h->profiling ? takeEvent(h) : nullptr;
        if (h->ph.precision == SPHGPU_PRECISION_MIXED) {
            launchGravityWalkMixed(h->s, h->tree, h->ph, h->d_lut_grav_f, h->d_err, st, e0, e1);
            h->launches += h->tree.walk_launches;
        } else {
            launchGravityWalk(h->s, h->tree, h->ph, h->d_lut_grav, h->d_err, st, e0, e1);
            h->launches += h->tree.walk_launches;
        }
        if (e0) {
            // (no walk was launched for an empty state: the events go back unrecorded)
            if (h->tree.walk_launches > 0) {
                h->marks.push_back({ SPHGPU_PHASE_WALK_EVALUATION, { e0, e1 } });
            } else {
                h->event_pool.push_back(e0);
                h->event_pool.push_back(e1);
            }
        }
    }
    h->gravity_current = true;
    return SPHGPU_OK;
}

sphgpu_status evalGravity(sphgpu_handle* h, cudaStream_t st) {
    const sphgpu_status s = evalGravityBuild(h, st);
    return s != SPHGPU_OK ? s : evalGravityWalk(h, st);
}

// materials initialize (EOS, rheology), neighbour grid and pair loop on the main stream; gravityInLoop: the
// pair loop adds s.agrav itself
void evalSphPrepare(sphgpu_handle* h) {
    {
        Phase ph(h, SPHGPU_PHASE_PREDICT);
        launchMaterialsInit(h->s, h->ph, h->d_mats, h->stream);
        h->launches += 1;
    }
    Phase ph(h, SPHGPU_PHASE_NEIGHBORS);
    // the mixed pair loop searches a grid of h_max cells
    launchGridBuild(h->s, h->grid, h->ph, h->stream, h->ph.precision == SPHGPU_PRECISION_MIXED);
    h->launches += h->grid.launches;
    launchGatherSorted(h->s, h->grid, h->ph, h->stream);
    h->launches += h->grid.launches;
}

void evalSphPairs(sphgpu_handle* h, bool gravityInLoop) {
    Phase ph(h, SPHGPU_PHASE_SPH_EVAL);
    Physics phs = h->ph;
    phs.gravity = gravityInLoop ? h->ph.gravity : 0;
    if (h->ph.correction) {
        // CorrectionTensor is a PRECOMPUTE derivative: every C_i before the velocity gradients
        if (h->ph.precision == SPHGPU_PRECISION_MIXED) {
            launchCorrectionMixed(h->s, h->grid, phs, h->d_lut_sph_f, h->stream);
        } else {
            launchCorrection64(h->s, h->grid, phs, h->d_lut_sph, h->stream);
        }
        h->launches += 1;
    }
    if (h->ph.precision == SPHGPU_PRECISION_MIXED) {
        launchPairSumMixed(h->s, h->grid, phs, h->d_mats, h->d_lut_sph_f, h->stream);
    } else {
        launchPairSum64(h->s, h->grid, phs, h->d_mats, h->d_lut_sph, h->stream);
    }
    h->launches += 1;
}

void evalSph(sphgpu_handle* h, bool gravityInLoop) {
    evalSphPrepare(h);
    evalSphPairs(h, gravityInLoop);
}

// ISolver::integrate on a state whose h is already clamped: materials initialize, gravity, pair loop,
// finalize. With self-gravity the order of GravitySolver::loop (core/sph/solvers/GravitySolver.cpp:64-91:
// gravity into the accumulator, then the pair loop) is kept in the arithmetic, not in time: the materials
// initialize and the pair loop (main stream) and the tree build + walk (gravity stream, higher priority; they
// read only positions, h and masses) run concurrently, and after both dv = a_gravity + a_sph: the same
// terms as the reference's accumulator, with the gravity term added after the pair sum instead of before it
// (a difference of rounding only).

sphgpu_status evalDerivatives(sphgpu_handle* h) {
    if (!h->ph.gravity) {
        evalSph(h, false);
        return SPHGPU_OK;
    }
    CUDA_TRY(h, cudaEventRecord(h->ev_fork, h->stream));
    CUDA_TRY(h, cudaStreamWaitEvent(h->gstream, h->ev_fork, 0));
    // The material update and the neighbour grid are queued before the tree build and run beside it; the pair loop
    // is queued once the build has returned to the host (it reads the level counts once at its end), so that it
    // runs beside the walk. The build is a chain of short dependent launches that the pair loop's blocks would
    // hold off the SMs. Measured on the 1.08M impact (ms per step): pair loop queued after the build 8.97, before
    // the build 9.50, after the walk's list phase (beside its evaluation alone) 9.36.
    evalSphPrepare(h);
    sphgpu_status st = evalGravityBuild(h, h->gstream);
    if (st != SPHGPU_OK) {
        return st;
    }
    evalSphPairs(h, false);
    st = evalGravityWalk(h, h->gstream);
    if (st != SPHGPU_OK) {
        return st;
    }
    CUDA_TRY(h, cudaEventRecord(h->ev_join, h->gstream));
    CUDA_TRY(h, cudaStreamWaitEvent(h->stream, h->ev_join, 0));
    {
        Phase ph(h, SPHGPU_PHASE_SPH_EVAL);
        launchAddGravity(h->s, h->stream);
        h->launches += 1;
    }
    return SPHGPU_OK;
}

// CachedGravity::evalSelfGravity (core/gravity/CachedGravity.h:45-63, wrapped around the gravity by
// Factory::getGravity for a positive GRAVITY_RECOMPUTATION_PERIOD, core/system/Factory.cpp:405-409): the
// accelerations of the last evaluation are reused while the run time is less than one period after it and the
// particle count is unchanged. Reads the run time from the device (one synchronisation per evaluation, with a
// positive period only).
sphgpu_status decideGravityCache(sphgpu_handle* h) {
    h->gravity_cached = false;
    const double period = h->cfg.gravity_recomputation_period;
    if (!(period > 0.) || !h->ph.gravity) {
        return SPHGPU_OK;
    }
    CUDA_TRY(h, cudaMemcpyAsync(h->h_pinned, h->d_time, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    const double t = *reinterpret_cast<const double*>(h->h_pinned);
    if (h->s.n == h->gravity_n_last && t - h->gravity_t_last < period) {
        h->gravity_cached = true;
    } else {
        h->gravity_t_last = t;
        h->gravity_n_last = h->s.n;
    }
    return SPHGPU_OK;
}

// HardSphereSolver::collide over [0, factor * dt) (dt on the device)
sphgpu_status collideNbody(sphgpu_handle* h, const double* dt, double factor) {
    Phase ph(h, SPHGPU_PHASE_COLLIDE);
    uint32_t capacityError = 0;
    const int st = nbodyCollide(h->s, h->grid, h->coll, h->cp, dt, factor, &capacityError, h->stream);
    h->launches += h->coll.launches;
    if (st == SPHGPU_ERR_CAPACITY) {
        // the collisions processed before the work space ran out are applied and their mergers removed
        h->gravity_current = false;
        return fail(h, SPHGPU_ERR_CAPACITY, "collision work space exhausted (bits 0x%x: 1 records, 2 heap, "
                                            "4 invalidated particles, 8 moved-particle lists)", capacityError);
    }
    if (st != SPHGPU_OK) {
        return cudaFail(h, cudaGetLastError(), "collide");
    }
    h->gravity_current = false;
    return SPHGPU_OK;
}

// HardSphereSolver::integrate, optionally followed by the leap-frog kick
sphgpu_status integrateNbody(sphgpu_handle* h, bool kick) {
    if (h->ph.gravity) {
        const sphgpu_status st = evalGravity(h, h->stream);
        if (st != SPHGPU_OK) {
            return st;
        }
    }
    Phase ph(h, SPHGPU_PHASE_CORRECT);
    launchNbodyIntegrate(h->s, h->ph.gravity != 0, h->d_dt, kick, h->stream);
    h->launches += 1;
    return SPHGPU_OK;
}

// LeapFrog::stepParticles with the N-body solver (core/timestepping/TimeStepping.cpp:352-391) and the
// acceleration criterion
sphgpu_status stepNbody(sphgpu_handle* h) {
    sphgpu_status st = collideNbody(h, h->d_dt, 0.5);
    if (st != SPHGPU_OK) {
        return st;
    }
    {
        Phase ph(h, SPHGPU_PHASE_PREDICT);
        launchNbodyDrift(h->s, h->ph, h->d_dt, h->d_dt_min, false, h->stream);
        h->launches += 1;
    }
    st = decideGravityCache(h);
    if (st != SPHGPU_OK) {
        return st;
    }
    st = integrateNbody(h, true);
    if (st != SPHGPU_OK) {
        return st;
    }
    st = collideNbody(h, h->d_dt, 0.5);
    if (st != SPHGPU_OK) {
        return st;
    }
    Phase ph(h, SPHGPU_PHASE_CORRECT);
    const bool criterion = (h->ph.criteria & SPHGPU_CRITERION_ACCELERATION) != 0;
    launchNbodyDrift(h->s, h->ph, h->d_dt, h->d_dt_min, criterion, h->stream);
    launchStepEnd(h->d_dt, h->d_dt_min, h->ph.max_dt, h->ph.max_change, h->d_time, criterion, h->stream);
    h->launches += 2;
    return SPHGPU_OK;
}

sphgpu_status requireSph(sphgpu_handle* h) {
    return h->ph.nbody ? fail(h, SPHGPU_ERR_UNSUPPORTED, "not available with the N-body solver") : SPHGPU_OK;
}

void swapPredictions(sphgpu_handle* h) {
    DState& s = h->s;
    std::swap(s.dv, s.pdv);
    std::swap(s.drho, s.pdrho);
    std::swap(s.du, s.pdu);
    std::swap(s.dS, s.pdS);
    std::swap(s.dD, s.pdD);
}

sphgpu_status validate(const sphgpu_config* c) {
    if (!c) {
        return fail(nullptr, SPHGPU_ERR_ARGUMENT, "config is NULL");
    }
    const bool nbody = c->solver_type == SPHGPU_SOLVER_NBODY_HARD_SPHERE;
    if (!nbody && (c->material_count == 0 || !c->materials)) {
        return fail(nullptr, SPHGPU_ERR_ARGUMENT, "at least one material is required");
    }
    if (c->material_count > 0 && !c->materials) {
        return fail(nullptr, SPHGPU_ERR_ARGUMENT, "materials is NULL");
    }
    if (!(c->gravity_recomputation_period >= 0.)) {
        return fail(nullptr, SPHGPU_ERR_ARGUMENT, "gravity_recomputation_period must not be negative");
    }
    if (c->gravity_kernel < SPHGPU_GRAVITY_KERNEL_POINT_PARTICLES ||
        c->gravity_kernel > SPHGPU_GRAVITY_KERNEL_SOLID_SPHERES) {
        return fail(nullptr, SPHGPU_ERR_UNSUPPORTED, "unknown gravity kernel %d", c->gravity_kernel);
    }
    if (c->gravity_leaf_size == 0 || c->gravity_leaf_size > 32) {
        return fail(nullptr, SPHGPU_ERR_UNSUPPORTED, "gravity_leaf_size must be in [1, 32] (got %u)",
            c->gravity_leaf_size);
    }
    if ((c->forces & SPHGPU_FORCE_SELF_GRAVITY) && !(c->gravity_opening_angle > 0.)) {
        return fail(nullptr, SPHGPU_ERR_ARGUMENT, "gravity_opening_angle must be positive");
    }
    if (c->gravity_multipole_order != 0 && c->gravity_multipole_order != 2 && c->gravity_multipole_order != 3) {
        return fail(nullptr, SPHGPU_ERR_UNSUPPORTED, "gravity_multipole_order must be 0, 2 or 3");
    }
    if (c->integrator != SPHGPU_INTEGRATOR_PREDICTOR_CORRECTOR && c->integrator != SPHGPU_INTEGRATOR_LEAP_FROG) {
        return fail(nullptr, SPHGPU_ERR_UNSUPPORTED, "unknown integrator %d", c->integrator);
    }
    if (c->precision != SPHGPU_PRECISION_FP64 && c->precision != SPHGPU_PRECISION_MIXED) {
        return fail(nullptr, SPHGPU_ERR_UNSUPPORTED, "unknown precision %d", c->precision);
    }
    if (c->precision == SPHGPU_PRECISION_MIXED && !nbody && c->particle_count >= NB_MAX_PARTICLES) {
        return fail(nullptr, SPHGPU_ERR_UNSUPPORTED, "the mixed-precision SPH path takes fewer than %u particles",
            NB_MAX_PARTICLES);
    }
    if (c->solver_type != SPHGPU_SOLVER_SYMMETRIC && c->solver_type != SPHGPU_SOLVER_ASYMMETRIC && !nbody) {
        return fail(nullptr, SPHGPU_ERR_UNSUPPORTED, "unknown solver type %d", c->solver_type);
    }
    if (nbody) {
        if (c->integrator != SPHGPU_INTEGRATOR_LEAP_FROG) {
            return fail(nullptr, SPHGPU_ERR_UNSUPPORTED, "the N-body solver is integrated by leap-frog only");
        }
        if (c->forces & ~uint32_t(SPHGPU_FORCE_SELF_GRAVITY)) {
            return fail(nullptr, SPHGPU_ERR_UNSUPPORTED, "the N-body solver has self-gravity as its only force");
        }
        if (c->timestep_criteria & ~uint32_t(SPHGPU_CRITERION_ACCELERATION)) {
            return fail(nullptr, SPHGPU_ERR_UNSUPPORTED,
                "the N-body solver supports the acceleration criterion only (0 = constant step)");
        }
        if ((c->timestep_criteria & SPHGPU_CRITERION_ACCELERATION) && !(c->derivative_factor > 0.)) {
            return fail(nullptr, SPHGPU_ERR_ARGUMENT, "derivative_factor must be positive");
        }
        if (c->collision_handler < SPHGPU_COLLISION_NONE || c->collision_handler > SPHGPU_COLLISION_MERGE_OR_BOUNCE) {
            return fail(nullptr, SPHGPU_ERR_UNSUPPORTED, "unknown collision handler %d", c->collision_handler);
        }
        if (c->overlap_handler < SPHGPU_OVERLAP_NONE || c->overlap_handler > SPHGPU_OVERLAP_PASS_OR_MERGE) {
            return fail(nullptr, SPHGPU_ERR_UNSUPPORTED, "unknown overlap handler %d", c->overlap_handler);
        }
        if (!(c->allowed_overlap >= 0.)) {
            return fail(nullptr, SPHGPU_ERR_ARGUMENT, "allowed_overlap must not be negative");
        }
        if (!(c->max_change >= 0.)) {
            return fail(nullptr, SPHGPU_ERR_ARGUMENT, "max_change must not be negative (0 = no limit)");
        }
        return SPHGPU_OK;
    }
    if (c->correction_tensor &&
        (c->solver_type != SPHGPU_SOLVER_ASYMMETRIC || !(c->forces & SPHGPU_FORCE_SOLID_STRESS))) {
        return fail(nullptr, SPHGPU_ERR_UNSUPPORTED,
            "the correction tensor needs the asymmetric solver and the solid stress force");
    }
    if (c->timestep_criteria & ~uint32_t(SPHGPU_CRITERION_ALL)) {
        return fail(nullptr, SPHGPU_ERR_UNSUPPORTED, "unknown time-step criterion bits 0x%x", c->timestep_criteria);
    }
    if ((c->timestep_criteria & (SPHGPU_CRITERION_DERIVATIVES | SPHGPU_CRITERION_ACCELERATION)) &&
        !(c->derivative_factor > 0.)) {
        return fail(nullptr, SPHGPU_ERR_ARGUMENT, "derivative_factor must be positive");
    }
    if ((c->timestep_criteria & SPHGPU_CRITERION_DIVERGENCE) && !(c->divergence_factor > 0.)) {
        return fail(nullptr, SPHGPU_ERR_ARGUMENT, "divergence_factor must be positive");
    }
    if (!(c->max_change >= 0.)) {
        return fail(nullptr, SPHGPU_ERR_ARGUMENT, "max_change must not be negative (0 = no limit)");
    }
    if (!(c->forces & SPHGPU_FORCE_PRESSURE)) {
        return fail(nullptr, SPHGPU_ERR_UNSUPPORTED, "the pressure force is required");
    }
    for (uint32_t k = 0; k < c->material_count; ++k) {
        const sphgpu_material& m = c->materials[k];
        if (m.eos != SPHGPU_EOS_TILLOTSON && m.eos != SPHGPU_EOS_IDEAL_GAS) {
            return fail(nullptr, SPHGPU_ERR_UNSUPPORTED, "material %u: unknown EOS %d", k, m.eos);
        }
        if (!(m.density > 0.)) {
            return fail(nullptr, SPHGPU_ERR_ARGUMENT, "material %u: density must be positive", k);
        }
    }
    return SPHGPU_OK;
}

} // namespace

extern "C" {

int sphgpu_abi_version(void) {
    return SPHGPU_ABI_VERSION;
}

const char* sphgpu_last_error(const sphgpu_handle* h) {
    return h ? h->error.c_str() : gCreateError.c_str();
}

sphgpu_status sphgpu_create(const sphgpu_config* config, sphgpu_handle** out) {
    if (!out) {
        return fail(nullptr, SPHGPU_ERR_ARGUMENT, "out is NULL");
    }
    *out = nullptr;
    sphgpu_status st = validate(config);
    if (st != SPHGPU_OK) {
        return st;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        return fail(nullptr, SPHGPU_ERR_CUDA, "no CUDA device available");
    }
    if (config->device < 0 || config->device >= ndev) {
        return fail(nullptr, SPHGPU_ERR_ARGUMENT, "device %d out of range", config->device);
    }
    if (cudaSetDevice(config->device) != cudaSuccess) {
        return fail(nullptr, SPHGPU_ERR_CUDA, "cudaSetDevice failed");
    }
    sphgpu_handle* h = new (std::nothrow) sphgpu_handle();
    if (!h) {
        return fail(nullptr, SPHGPU_ERR_ALLOCATION, "host allocation failed");
    }
    h->cfg = *config;
    h->materials.assign(config->materials, config->materials + config->material_count);
    h->cfg.materials = h->materials.data();
    const uint32_t n = config->particle_count;

    Physics& ph = h->ph;
    std::memset(&ph, 0, sizeof(ph));
    bool anyRheology = false, anyDamage = false;
    for (const sphgpu_material& m : h->materials) {
        anyRheology = anyRheology || m.yielding != SPHGPU_YIELDING_NONE;
        anyDamage = anyDamage || (m.yielding != SPHGPU_YIELDING_NONE && m.damage != SPHGPU_DAMAGE_NONE);
    }
    ph.solid = (config->forces & SPHGPU_FORCE_SOLID_STRESS) ? 1 : 0;
    ph.damage = ph.solid && anyDamage ? 1 : 0;
    ph.gravity = (config->forces & SPHGPU_FORCE_SELF_GRAVITY) ? 1 : 0;
    ph.adaptive_h = config->adaptive_smoothing_length ? 1 : 0;
    ph.sum_only_undamaged = config->sum_only_undamaged ? 1 : 0;
    ph.integrator = config->integrator;
    ph.precision = config->precision;
    ph.multipole_order = config->gravity_multipole_order;
    ph.kernel_radius = config->gravity_kernel == SPHGPU_GRAVITY_KERNEL_POINT_PARTICLES ? 0 : 2;
    ph.leaf_size = config->gravity_leaf_size;
    ph.nmat = config->material_count;
    ph.h_lo = config->smoothing_length_range[0];
    ph.h_hi = config->smoothing_length_range[1];
    ph.av_alpha = config->av_alpha;
    ph.av_beta = config->av_beta;
    ph.G = config->gravity_constant;
    ph.theta_inv = config->gravity_opening_angle > 0. ? 1. / config->gravity_opening_angle : 2.;
    ph.courant = config->courant_number;
    ph.max_dt = config->max_timestep;
    ph.nbody = config->solver_type == SPHGPU_SOLVER_NBODY_HARD_SPHERE ? 1 : 0;
    ph.criteria = config->timestep_criteria || ph.nbody ? config->timestep_criteria
                                                         : uint32_t(SPHGPU_CRITERION_COURANT);
    ph.derivative_factor = config->derivative_factor;
    ph.divergence_factor = config->divergence_factor;
    ph.max_change = config->max_change > 0. ? config->max_change : DBL_MAX;
    ph.correction = config->correction_tensor ? 1 : 0;
    (void)anyRheology;
    CollideParams& cp = h->cp;
    std::memset(&cp, 0, sizeof(cp));
    cp.handler = config->collision_handler;
    cp.overlap = config->overlap_handler;
    cp.rest_n = config->restitution_normal;
    cp.rest_t = config->restitution_tangent;
    cp.allowed = config->allowed_overlap;
    cp.bounce_limit = config->bounce_merge_limit;
    cp.rotation_limit = config->rotation_merge_limit;
    cp.max_bounces = config->max_bounces;

    cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) {
        int leastPriority = 0, greatestPriority = 0;
        e = cudaDeviceGetStreamPriorityRange(&leastPriority, &greatestPriority);
        if (e == cudaSuccess) {
            e = cudaStreamCreateWithPriority(&h->gstream, cudaStreamNonBlocking, greatestPriority);
        }
    }
    if (e == cudaSuccess) {
        e = cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming);
    }
    if (e == cudaSuccess) {
        e = cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming);
    }

    DState& s = h->s;
    s.n = n;
    const size_t nn = std::max<uint32_t>(n, 1);
    auto A = [&](auto** p, size_t count) {
        if (e == cudaSuccess) {
            e = devAlloc(h, p, count);
        }
    };
    A(&s.r, nn);
    A(&s.v, nn);
    A(&s.dv, nn);
    A(&s.agrav, nn);
    A(&s.m, nn);
    A(&s.u, nn);
    if (ph.nbody) {
        // HardSphereSolver state: r (radius as h), v, dv, m, angular frequency; u stays 0 for the totals
        A(&s.omega, nn);
        A(&h->coll.tmp_r, nn);
        A(&h->coll.tmp_v, nn);
        A(&h->coll.tmp_dv, nn);
        A(&h->coll.tmp_w, nn);
        A(&h->coll.tmp_m, nn);
        A(&s.origin, nn);
        A(&h->coll.tmp_origin, nn);
        A(&h->d_dtc, 1);
    } else {
        A(&s.pdv, nn);
        A(&s.rho, nn);
        A(&s.drho, nn);
        A(&s.pdrho, nn);
        A(&s.du, nn);
        A(&s.pdu, nn);
        A(&s.p, nn);
        A(&s.cs, nn);
        A(&s.divv, nn);
        A(&s.ncnt, nn);
        A(&s.flag, nn);
        A(&s.mat, nn);
    }
    if (ph.solid) {
        A(&s.S, 5 * nn);
        A(&s.dS, 5 * nn);
        A(&s.pdS, 5 * nn);
        A(&s.gradv, 6 * nn);
        if (ph.correction) {
            A(&s.corr, 6 * nn);
        }
        A(&s.reduce, nn);
    }
    if (ph.damage) {
        A(&s.D, nn);
        A(&s.dD, nn);
        A(&s.pdD, nn);
        A(&s.eps_min, nn);
        A(&s.m_zero, nn);
        A(&s.growth, nn);
        A(&s.n_flaws, nn);
    }
    A(&h->d_mats, std::max<size_t>(h->materials.size(), 1));
    A(&h->d_lut_sph, LUT_ENTRIES + 1);
    A(&h->d_lut_grav, LUT_ENTRIES + 1);
    A(&h->d_lut_sph_f, LUT_ENTRIES + 1);
    A(&h->d_lut_grav_f, LUT_ENTRIES + 1);
    A(&h->d_dt, 1);
    A(&h->d_dt_min, 1);
    A(&h->d_time, 1);
    A(&h->d_err, 1);
    A(&h->d_tot_partial, 256 * 9);
    A(&h->d_tot, 9);
    A(&h->d_count, 2);
    if (e == cudaSuccess) {
        e = cudaMallocHost((void**)&h->h_pinned, 64 * sizeof(unsigned long long));
    }
    if (e == cudaSuccess) {
        e = gridAllocate(h->grid, n, ph.solid != 0, ph.correction != 0, !ph.nbody,
            !ph.nbody && ph.precision == SPHGPU_PRECISION_MIXED);
    }
    if (e == cudaSuccess && ph.gravity) {
        e = treeAllocate(h->tree, n, ph.leaf_size);
    }
    if (e == cudaSuccess && ph.nbody) {
        e = collideAllocate(h->coll, n, h->grid.cell_capacity, config->collision_records);
    }
    if (e != cudaSuccess) {
        const std::string msg = std::string("device allocation failed: ") + cudaGetErrorString(e);
        sphgpu_destroy(h);
        cudaGetLastError();
        return fail(nullptr, SPHGPU_ERR_ALLOCATION, "%s", msg.c_str());
    }
    std::vector<MaterialD> md;
    for (const sphgpu_material& m : h->materials) {
        md.push_back(toDevice(m));
    }
    const std::vector<double> lutS = makeLut(cubicGrad);
    // LutKernel<3> of the gravity kernel: GravityKernel<CubicSpline<3>>, or SolidSphereKernel, whose gradImpl
    // is 1 everywhere (core/sph/kernel/GravityKernel.h:121-136)
    const std::vector<double> lutG = config->gravity_kernel == SPHGPU_GRAVITY_KERNEL_SOLID_SPHERES
                                         ? makeLut([](double) { return 1.; })
                                         : makeLut(gravGrad);
    std::vector<float> lutSf(lutS.begin(), lutS.end());
    std::vector<float> lutGf(lutG.begin(), lutG.end());
    const double dt0 = config->initial_timestep;
    const double big = 1.7976931348623157e308;
    e = cudaMemcpy(h->d_mats, md.data(), md.size() * sizeof(MaterialD), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        e = cudaMemcpy(h->d_lut_sph, lutS.data(), lutS.size() * sizeof(double), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) {
        e = cudaMemcpy(h->d_lut_grav, lutG.data(), lutG.size() * sizeof(double), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) {
        e = cudaMemcpy(h->d_lut_sph_f, lutSf.data(), lutSf.size() * sizeof(float), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) {
        e = cudaMemcpy(h->d_lut_grav_f, lutGf.data(), lutGf.size() * sizeof(float), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) {
        e = cudaMemcpy(h->d_dt, &dt0, sizeof(double), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) {
        e = cudaMemcpy(h->d_dt_min, &big, sizeof(double), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) {
        e = cudaMemset(s.u, 0, nn * sizeof(double));
    }
    if (e == cudaSuccess) {
        e = cudaMemset(h->d_time, 0, sizeof(double));
    }
    if (e == cudaSuccess && s.omega) {
        // HardSphereSolver::create inserts ANGULAR_FREQUENCY = 0 (core/gravity/NBodySolver.cpp:487-490)
        e = cudaMemset(s.omega, 0, nn * sizeof(dbl4));
    }
    if (e == cudaSuccess && s.origin) {
        launchIota(s.origin, n, nullptr);
        e = cudaGetLastError();
        h->n_sync = n;
    }
    if (e == cudaSuccess) {
        // reference defaults: every particle has STRESS_REDUCING = 1 (VonMisesRheology::create)
        if (s.reduce) {
            std::vector<double> ones(nn, 1.);
            e = cudaMemcpy(s.reduce, ones.data(), nn * sizeof(double), cudaMemcpyHostToDevice);
        }
    }
    if (e == cudaSuccess) {
        e = cudaDeviceSynchronize();
    }
    if (e != cudaSuccess) {
        const std::string msg = cudaGetErrorString(e);
        sphgpu_destroy(h);
        return fail(nullptr, SPHGPU_ERR_CUDA, "initialisation failed: %s", msg.c_str());
    }
    *out = h;
    return SPHGPU_OK;
}

sphgpu_status sphgpu_destroy(sphgpu_handle* h) {
    if (!h) {
        return SPHGPU_OK;
    }
    if (h->stream) {
        cudaStreamSynchronize(h->stream);
    }
    for (void* p : h->allocations) {
        cudaFree(p);
    }
    for (auto& m : h->marks) {
        cudaEventDestroy(m.second.first);
        cudaEventDestroy(m.second.second);
    }
    for (cudaEvent_t e : h->event_pool) {
        cudaEventDestroy(e);
    }
    gridFree(h->grid);
    treeFree(h->tree);
    collideFree(h->coll);
    adjointFree(h->adjoint);
    if (h->h_pinned) {
        cudaFreeHost(h->h_pinned);
    }
    if (h->gstream) {
        cudaStreamSynchronize(h->gstream);
        cudaStreamDestroy(h->gstream);
    }
    if (h->ev_fork) {
        cudaEventDestroy(h->ev_fork);
    }
    if (h->ev_join) {
        cudaEventDestroy(h->ev_join);
    }

    if (h->stream) {
        cudaStreamDestroy(h->stream);
    }
    delete h;
    return SPHGPU_OK;
}

void* sphgpu_stream(sphgpu_handle* h) {
    return h ? (void*)h->stream : nullptr;
}

sphgpu_status sphgpu_synchronize(sphgpu_handle* h) {
    if (!h) {
        return SPHGPU_ERR_ARGUMENT;
    }
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return SPHGPU_OK;
}

sphgpu_status sphgpu_set_quantity(sphgpu_handle* h, int32_t id, int32_t order, const void* src, uint64_t count) {
    if (!h || !src) {
        return h ? fail(h, SPHGPU_ERR_ARGUMENT, "NULL source") : SPHGPU_ERR_ARGUMENT;
    }
    QuantitySlot q;
    if (!slotOf(h, id, order, q)) {
        return fail(h, SPHGPU_ERR_ARGUMENT, "unknown quantity %d (order %d)", id, order);
    }
    if (!q.dev) {
        return fail(h, SPHGPU_ERR_ARGUMENT, "quantity %d is not used by the configured physics", id);
    }
    if (count != h->s.n) {
        return fail(h, SPHGPU_ERR_ARGUMENT, "quantity %d: %llu values given for %u particles", id,
            (unsigned long long)count, h->s.n);
    }
    if (id == SPHGPU_Q_POSITION && order == 0) {
        h->grid_current = false;
    }
    const size_t n = count;
    if (q.soa) {
        const double* a = static_cast<const double*>(src);
        std::vector<double> t(n * q.comps);
        for (size_t i = 0; i < n; ++i) {
            for (int c = 0; c < q.comps; ++c) {
                t[c * n + i] = a[i * q.comps + c];
            }
        }
        CUDA_TRY(h, cudaMemcpyAsync(q.dev, t.data(), t.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    } else {
        CUDA_TRY(h, cudaMemcpyAsync(q.dev, src, n * q.comps * q.bytes, cudaMemcpyHostToDevice, h->stream));
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    }
    h->gravity_current = false;
    if (h->s.origin && id == SPHGPU_Q_POSITION && order == 0) {
        // a new state: removals are reported relative to it
        launchIota(h->s.origin, h->s.n, h->stream);
        CUDA_TRY(h, cudaGetLastError());
        h->n_sync = h->s.n;
    }
    return SPHGPU_OK;
}

sphgpu_status sphgpu_get_quantity(sphgpu_handle* h, int32_t id, int32_t order, void* dst, uint64_t count) {
    if (!h || !dst) {
        return h ? fail(h, SPHGPU_ERR_ARGUMENT, "NULL destination") : SPHGPU_ERR_ARGUMENT;
    }
    QuantitySlot q;
    if (!slotOf(h, id, order, q) || !q.dev) {
        return fail(h, SPHGPU_ERR_ARGUMENT, "quantity %d (order %d) is not held by this handle", id, order);
    }
    if (count != h->s.n) {
        return fail(h, SPHGPU_ERR_ARGUMENT, "quantity %d: room for %llu values, %u particles", id,
            (unsigned long long)count, h->s.n);
    }
    const size_t n = count;
    if (q.soa) {
        std::vector<double> t(n * q.comps);
        CUDA_TRY(h, cudaMemcpyAsync(t.data(), q.dev, t.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
        double* a = static_cast<double*>(dst);
        for (size_t i = 0; i < n; ++i) {
            for (int c = 0; c < q.comps; ++c) {
                a[i * q.comps + c] = t[c * n + i];
            }
        }
    } else {
        CUDA_TRY(h, cudaMemcpyAsync(dst, q.dev, n * q.comps * q.bytes, cudaMemcpyDeviceToHost, h->stream));
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    }
    return SPHGPU_OK;
}

sphgpu_status sphgpu_build_neighbors(sphgpu_handle* h) {
    if (!h) {
        return SPHGPU_ERR_ARGUMENT;
    }
    if (requireSph(h) != SPHGPU_OK) {
        return SPHGPU_ERR_UNSUPPORTED;
    }
    launchGridBuild(h->s, h->grid, h->ph, h->stream);
    launchGatherSorted(h->s, h->grid, h->ph, h->stream);
    CUDA_TRY(h, cudaGetLastError());
    h->grid_current = true;
    return SPHGPU_OK;
}

sphgpu_status sphgpu_find_neighbors(sphgpu_handle* h, const double pos[3], double radius, uint32_t* indices,
    double* dist_sqr, uint64_t capacity, uint64_t* count) {
    if (!h || !pos || !count || (capacity && (!indices || !dist_sqr)) || !(radius >= 0.)) {
        return h ? fail(h, SPHGPU_ERR_ARGUMENT, "invalid query arguments") : SPHGPU_ERR_ARGUMENT;
    }
    if (!h->grid_current) {
        return fail(h, SPHGPU_ERR_STATE, "find_neighbors needs sphgpu_build_neighbors of the current positions");
    }
    const uint64_t cap = std::min<uint64_t>(capacity, h->s.n);
    uint32_t* di = nullptr;
    double* dd = nullptr;
    cudaError_t e = cudaSuccess;
    if (cap) {
        e = cudaMalloc(&di, cap * sizeof(uint32_t));
        if (e == cudaSuccess) {
            e = cudaMalloc(&dd, cap * sizeof(double));
        }
    }
    const dbl4 p = mkd4(pos[0], pos[1], pos[2], 0.);
    if (e == cudaSuccess) {
        launchFindBall(h->grid, h->s.n, p, radius, di, dd, h->d_count, cap, h->stream);
        h->launches += 1;
        e = cudaMemcpyAsync(h->h_pinned, h->d_count, sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->stream);
    }
    if (e == cudaSuccess) {
        e = cudaStreamSynchronize(h->stream);
    }
    const uint64_t total = e == cudaSuccess ? h->h_pinned[0] : 0;
    std::vector<uint32_t> idx;
    std::vector<double> d2;
    if (e == cudaSuccess && total <= capacity && total > 0) {
        idx.resize(total);
        d2.resize(total);
        e = cudaMemcpy(idx.data(), di, total * sizeof(uint32_t), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) {
            e = cudaMemcpy(d2.data(), dd, total * sizeof(double), cudaMemcpyDeviceToHost);
        }
    }
    cudaFree(di);
    cudaFree(dd);
    if (e != cudaSuccess) {
        return cudaFail(h, e, "find neighbors");
    }
    *count = total;
    if (total > capacity) {
        return fail(h, SPHGPU_ERR_CAPACITY, "%llu neighbours, capacity %llu", (unsigned long long)total,
            (unsigned long long)capacity);
    }
    // ascending particle index (the device emits them unordered)
    std::vector<uint64_t> order(total);
    for (uint64_t k = 0; k < total; ++k) {
        order[k] = k;
    }
    std::sort(order.begin(), order.end(), [&](uint64_t a, uint64_t b) { return idx[a] < idx[b]; });
    for (uint64_t k = 0; k < total; ++k) {
        indices[k] = idx[order[k]];
        dist_sqr[k] = d2[order[k]];
    }
    return SPHGPU_OK;
}

namespace {

sphgpu_status listPairs(sphgpu_handle* h, bool directed, uint32_t* pair_i, uint32_t* pair_j, uint64_t capacity,
    uint64_t* npairs);

} // namespace

sphgpu_status sphgpu_get_pairs(sphgpu_handle* h, uint32_t* pair_i, uint32_t* pair_j, uint64_t capacity,
    uint64_t* npairs) {
    return listPairs(h, false, pair_i, pair_j, capacity, npairs);
}

sphgpu_status sphgpu_get_radius_pairs(sphgpu_handle* h, uint32_t* pair_i, uint32_t* pair_j, uint64_t capacity,
    uint64_t* npairs) {
    return listPairs(h, true, pair_i, pair_j, capacity, npairs);
}

namespace {

sphgpu_status listPairs(sphgpu_handle* h, bool directed, uint32_t* pair_i, uint32_t* pair_j, uint64_t capacity,
    uint64_t* npairs) {
    if (!h || !npairs || (capacity && (!pair_i || !pair_j))) {
        return h ? fail(h, SPHGPU_ERR_ARGUMENT, "invalid pair buffers") : SPHGPU_ERR_ARGUMENT;
    }
    const sphgpu_status st = sphgpu_build_neighbors(h);
    if (st != SPHGPU_OK) {
        return st;
    }
    if (directed) {
        launchRadiusPairs(h->s, h->grid, nullptr, nullptr, h->d_count, 0, h->stream);
    } else {
        launchCountPairs(h->s, h->grid, h->d_count, h->stream);
    }
    CUDA_TRY(h, cudaMemcpyAsync(h->h_pinned, h->d_count, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
        h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    const unsigned long long total = h->h_pinned[0];
    *npairs = total;
    if (total > capacity) {
        return fail(h, SPHGPU_ERR_CAPACITY, "%llu pairs, capacity %llu", total, (unsigned long long)capacity);
    }
    if (total == 0) {
        return SPHGPU_OK;
    }
    uint32_t* dpi = nullptr;
    uint32_t* dpj = nullptr;
    CUDA_TRY(h, cudaMalloc(&dpi, total * sizeof(uint32_t)));
    cudaError_t e = cudaMalloc(&dpj, total * sizeof(uint32_t));
    if (e != cudaSuccess) {
        cudaFree(dpi);
        return cudaFail(h, e, "pair buffer");
    }
    if (directed) {
        launchRadiusPairs(h->s, h->grid, dpi, dpj, h->d_count, total, h->stream);
    } else {
        launchListPairs(h->s, h->grid, dpi, dpj, h->d_count, total, h->stream);
    }
    std::vector<uint32_t> a(total), b(total);
    e = cudaMemcpyAsync(a.data(), dpi, total * sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) {
        e = cudaMemcpyAsync(b.data(), dpj, total * sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream);
    }
    if (e == cudaSuccess) {
        e = cudaStreamSynchronize(h->stream);
    }
    cudaFree(dpi);
    cudaFree(dpj);
    if (e != cudaSuccess) {
        return cudaFail(h, e, "pair list");
    }
    std::vector<uint64_t> key(total);
    for (size_t k = 0; k < total; ++k) {
        key[k] = (uint64_t(a[k]) << 32) | b[k];
    }
    std::sort(key.begin(), key.end());
    for (size_t k = 0; k < total; ++k) {
        pair_i[k] = uint32_t(key[k] >> 32);
        pair_j[k] = uint32_t(key[k] & 0xffffffffu);
    }
    return SPHGPU_OK;
}

} // namespace

sphgpu_status sphgpu_gravity_build(sphgpu_handle* h) {
    if (!h) {
        return SPHGPU_ERR_ARGUMENT;
    }
    if (!h->ph.gravity) {
        return fail(h, SPHGPU_ERR_STATE, "self-gravity is not enabled in the configuration");
    }
    {
        Phase ph(h, SPHGPU_PHASE_GRAVITY_BUILD);
        cudaError_t e = treeBuild(h->s, h->tree, h->ph, h->d_err, h->stream);
        if (e != cudaSuccess) {
            return cudaFail(h, e, "gravity build");
        }
        h->launches += h->tree.launches;
    }
    return checkDeviceError(h);
}

sphgpu_status sphgpu_gravity_eval(sphgpu_handle* h, double* dv, uint64_t count) {
    if (!h) {
        return SPHGPU_ERR_ARGUMENT;
    }
    if (!h->ph.gravity || !h->tree.built) {
        return fail(h, SPHGPU_ERR_STATE, "gravity_eval before gravity_build");
    }
    if (dv && count != h->s.n) {
        return fail(h, SPHGPU_ERR_ARGUMENT, "dv holds %llu particles, state has %u", (unsigned long long)count,
            h->s.n);
    }
    // the walk, again with check lists four times as long when one outgrew them (small opening angles)
    for (int attempt = 0;; ++attempt) {
        {
            Phase ph(h, SPHGPU_PHASE_GRAVITY_EVAL);
            if (h->ph.precision == SPHGPU_PRECISION_MIXED) {
                launchGravityWalkMixed(h->s, h->tree, h->ph, h->d_lut_grav_f, h->d_err, h->stream);
                h->launches += h->tree.walk_launches;
            } else {
                launchGravityWalk(h->s, h->tree, h->ph, h->d_lut_grav, h->d_err, h->stream);
                h->launches += h->tree.walk_launches;
            }
        }
        CUDA_TRY(h, cudaGetLastError());
        CUDA_TRY(h, cudaMemcpyAsync(h->h_pinned, h->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
        const uint32_t bits = *reinterpret_cast<uint32_t*>(h->h_pinned);
        if (bits == uint32_t(DEV_ERR_WALK_CAPACITY) && attempt < 3) {
            CUDA_TRY(h, cudaMemsetAsync(h->d_err, 0, sizeof(uint32_t), h->stream));
            CUDA_TRY(h, treeGrowWalkScratch(h->tree, 4 * h->tree.walk_capacity));
            continue;
        }
        break;
    }
    const sphgpu_status st = checkDeviceError(h);
    if (st != SPHGPU_OK) {
        return st;
    }
    if (dv) {
        std::vector<double> a(size_t(h->s.n) * 4);
        CUDA_TRY(h, cudaMemcpyAsync(a.data(), h->s.agrav, a.size() * sizeof(double), cudaMemcpyDeviceToHost,
            h->stream));
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
        for (size_t i = 0; i < size_t(h->s.n); ++i) {
            for (int c = 0; c < 3; ++c) {
                dv[4 * i + c] += a[4 * i + c];
            }
        }
    }
    return SPHGPU_OK;
}

sphgpu_status sphgpu_gravity_attractors(sphgpu_handle* h, const double* attractors, uint64_t count,
    double* attractor_acc, double* dv, uint64_t dv_count) {
    if (!h || (count && (!attractors || !attractor_acc)) || (dv && dv_count != h->s.n) || count > 0xffffull) {
        return h ? fail(h, SPHGPU_ERR_ARGUMENT, "invalid attractor or acceleration buffers") : SPHGPU_ERR_ARGUMENT;
    }
    if (!h->ph.gravity) {
        return fail(h, SPHGPU_ERR_STATE, "gravity_attractors without self-gravity");
    }
    if (count == 0) {
        return SPHGPU_OK;
    }
    const uint32_t n = h->s.n;
    const size_t partials = gravityAttractorPartials(n, uint32_t(count));
    double* dAtt = nullptr;
    double* dAcc = nullptr;
    double* dPart = nullptr;
    dbl4* dDv = nullptr;
    cudaError_t e = cudaMalloc(&dAtt, 5 * count * sizeof(double));
    if (e == cudaSuccess) {
        e = cudaMalloc(&dAcc, 3 * count * sizeof(double));
    }
    if (e == cudaSuccess && partials) {
        e = cudaMalloc(&dPart, partials * sizeof(double));
    }
    if (e == cudaSuccess && n) {
        e = cudaMalloc(&dDv, size_t(n) * sizeof(dbl4));
    }
    if (e == cudaSuccess) {
        e = cudaMemcpyAsync(dAtt, attractors, 5 * count * sizeof(double), cudaMemcpyHostToDevice, h->stream);
    }
    if (e == cudaSuccess) {
        e = cudaMemcpyAsync(dAcc, attractor_acc, 3 * count * sizeof(double), cudaMemcpyHostToDevice, h->stream);
    }
    if (e == cudaSuccess && n) {
        e = dv ? cudaMemcpyAsync(dDv, dv, size_t(n) * sizeof(dbl4), cudaMemcpyHostToDevice, h->stream)
               : cudaMemsetAsync(dDv, 0, size_t(n) * sizeof(dbl4), h->stream);
    }
    if (e == cudaSuccess) {
        launchGravityAttractors(h->s, h->ph, h->d_lut_grav, dAtt, uint32_t(count), dDv, dPart, dAcc, h->stream);
        h->launches += 2;
        e = cudaMemcpyAsync(attractor_acc, dAcc, 3 * count * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    }
    if (e == cudaSuccess && dv && n) {
        e = cudaMemcpyAsync(dv, dDv, size_t(n) * sizeof(dbl4), cudaMemcpyDeviceToHost, h->stream);
    }
    if (e == cudaSuccess) {
        e = cudaStreamSynchronize(h->stream);
    }
    for (void* p : { (void*)dAtt, (void*)dAcc, (void*)dPart, (void*)dDv }) {
        if (p) {
            cudaFree(p);
        }
    }
    if (e != cudaSuccess) {
        return cudaFail(h, e, "gravity attractors");
    }
    return SPHGPU_OK;
}

sphgpu_status sphgpu_gravity_direct(sphgpu_handle* h, const uint32_t* targets, uint64_t ntargets, double* acc) {
    if (!h || (ntargets && (!targets || !acc)) || ntargets > 0xffffffffull) {
        return h ? fail(h, SPHGPU_ERR_ARGUMENT, "invalid target buffers") : SPHGPU_ERR_ARGUMENT;
    }
    if (!h->ph.gravity) {
        return fail(h, SPHGPU_ERR_STATE, "gravity_direct without self-gravity");
    }
    for (uint64_t k = 0; k < ntargets; ++k) {
        if (targets[k] >= h->s.n) {
            return fail(h, SPHGPU_ERR_ARGUMENT, "target %llu out of range", (unsigned long long)targets[k]);
        }
    }
    if (ntargets == 0) {
        return SPHGPU_OK;
    }
    uint32_t* dt = nullptr;
    dbl4* da = nullptr;
    CUDA_TRY(h, cudaMalloc(&dt, ntargets * sizeof(uint32_t)));
    cudaError_t e = cudaMalloc(&da, ntargets * sizeof(dbl4));
    if (e == cudaSuccess) {
        e = cudaMemcpyAsync(dt, targets, ntargets * sizeof(uint32_t), cudaMemcpyHostToDevice, h->stream);
    }
    if (e == cudaSuccess) {
        launchGravityDirect(h->s, h->ph, h->d_lut_grav, dt, uint32_t(ntargets), da, h->stream);
        e = cudaMemcpyAsync(acc, da, ntargets * sizeof(dbl4), cudaMemcpyDeviceToHost, h->stream);
    }
    if (e == cudaSuccess) {
        e = cudaStreamSynchronize(h->stream);
    }
    cudaFree(dt);
    if (da) {
        cudaFree(da);
    }
    if (e != cudaSuccess) {
        return cudaFail(h, e, "gravity direct");
    }
    return SPHGPU_OK;
}

sphgpu_status sphgpu_gravity_eval_points(sphgpu_handle* h, const double* points, uint64_t npoints, double* acc) {
    if (!h || (npoints && (!points || !acc))) {
        return h ? fail(h, SPHGPU_ERR_ARGUMENT, "invalid point buffers") : SPHGPU_ERR_ARGUMENT;
    }
    if (!h->ph.gravity || !h->tree.built) {
        return fail(h, SPHGPU_ERR_STATE, "gravity_eval_points before gravity_build");
    }
    if (npoints == 0) {
        return SPHGPU_OK;
    }
    dbl4* dp = nullptr;
    dbl4* da = nullptr;
    CUDA_TRY(h, cudaMalloc(&dp, npoints * sizeof(dbl4)));
    cudaError_t e = cudaMalloc(&da, npoints * sizeof(dbl4));
    if (e == cudaSuccess) {
        e = cudaMemcpyAsync(dp, points, npoints * sizeof(dbl4), cudaMemcpyHostToDevice, h->stream);
    }
    if (e == cudaSuccess) {
        treeEnsureFp64Moments(h->s, h->tree, h->ph, h->stream);
        launchGravityPoints(h->s, h->tree, h->ph, h->d_lut_grav, dp, da, uint32_t(npoints), h->stream);
        e = cudaMemcpyAsync(acc, da, npoints * sizeof(dbl4), cudaMemcpyDeviceToHost, h->stream);
    }
    if (e == cudaSuccess) {
        e = cudaStreamSynchronize(h->stream);
    }
    cudaFree(dp);
    if (da) {
        cudaFree(da);
    }
    if (e != cudaSuccess) {
        return cudaFail(h, e, "gravity points");
    }
    return SPHGPU_OK;
}

sphgpu_status sphgpu_gravity_stats(sphgpu_handle* h, uint64_t out[3]) {
    if (!h || !out) {
        return SPHGPU_ERR_ARGUMENT;
    }
    if (!h->ph.gravity) {
        return fail(h, SPHGPU_ERR_STATE, "self-gravity is not enabled");
    }
    CUDA_TRY(h, cudaMemcpyAsync(h->h_pinned, h->tree.stats, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
        h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    out[0] = h->h_pinned[0];
    out[1] = h->h_pinned[1];
    out[2] = h->tree.node_count;
    return SPHGPU_OK;
}

sphgpu_status sphgpu_gravity_interactions(sphgpu_handle* h, uint64_t out[2]) {
    if (!h || !out) {
        return SPHGPU_ERR_ARGUMENT;
    }
    if (!h->ph.gravity) {
        return fail(h, SPHGPU_ERR_STATE, "self-gravity is not enabled");
    }
    CUDA_TRY(h, cudaMemcpyAsync(h->h_pinned, h->tree.stats + 2, 2 * sizeof(unsigned long long),
        cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    out[0] = h->h_pinned[0];
    out[1] = h->h_pinned[1];
    return SPHGPU_OK;
}

sphgpu_status sphgpu_integrate(sphgpu_handle* h) {
    if (!h) {
        return SPHGPU_ERR_ARGUMENT;
    }
    h->grid_current = false;
    const sphgpu_status cst = decideGravityCache(h);
    if (cst != SPHGPU_OK) {
        return cst;
    }
    if (h->ph.nbody) {
        const sphgpu_status st = integrateNbody(h, false);
        if (st != SPHGPU_OK) {
            return st;
        }
        CUDA_TRY(h, cudaGetLastError());
        return checkDeviceError(h);
    }
    {
        Phase ph(h, SPHGPU_PHASE_PREDICT);
        if (launchClampH(h->s, h->ph, h->stream)) {
            h->launches += 1;
        }
    }
    sphgpu_status st = evalDerivatives(h);
    if (st != SPHGPU_OK) {
        return st;
    }
    CUDA_TRY(h, cudaGetLastError());
    return checkDeviceError(h);
}

sphgpu_status sphgpu_step(sphgpu_handle* h, uint32_t nsteps) {
    if (!h) {
        return SPHGPU_ERR_ARGUMENT;
    }
    h->grid_current = false;
    for (uint32_t k = 0; k < nsteps; ++k) {
        if (h->ph.nbody) {
            const sphgpu_status st = stepNbody(h);
            if (st != SPHGPU_OK) {
                return st;
            }
            CUDA_TRY(h, cudaGetLastError());
            continue;
        }
        const bool lf = h->ph.integrator == SPHGPU_INTEGRATOR_LEAP_FROG;
        {
            const sphgpu_status cst = decideGravityCache(h);
            if (cst != SPHGPU_OK) {
                return cst;
            }
        }
        {
            Phase ph(h, SPHGPU_PHASE_PREDICT);
            if (lf) {
                launchLeapFrogDriftInit(h->s, h->ph, h->d_mats, h->d_dt, h->stream);
            } else {
                launchPredict(h->s, h->ph, h->d_mats, h->d_dt, h->stream);
                swapPredictions(h);
            }
            h->launches += 1;
        }
        sphgpu_status st = evalDerivatives(h);
        if (st != SPHGPU_OK) {
            return st;
        }
        {
            Phase ph(h, SPHGPU_PHASE_CORRECT);
            if (lf) {
                launchLeapFrogKick(h->s, h->ph, h->d_mats, h->d_dt, h->d_dt_min, h->stream);
            } else {
                launchCorrect(h->s, h->ph, h->d_mats, h->d_dt, h->d_dt_min, h->stream);
            }
            launchStepEnd(h->d_dt, h->d_dt_min, h->ph.max_dt, h->ph.max_change, h->d_time, true, h->stream);
            h->launches += 2;
        }
        CUDA_TRY(h, cudaGetLastError());
    }
    return checkDeviceError(h);
}

sphgpu_status sphgpu_get_timestep(sphgpu_handle* h, double* dt) {
    if (!h || !dt) {
        return SPHGPU_ERR_ARGUMENT;
    }
    CUDA_TRY(h, cudaMemcpyAsync(dt, h->d_dt, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return SPHGPU_OK;
}

sphgpu_status sphgpu_set_timestep(sphgpu_handle* h, double dt) {
    if (!h || !(dt > 0.)) {
        return h ? fail(h, SPHGPU_ERR_ARGUMENT, "time step must be positive") : SPHGPU_ERR_ARGUMENT;
    }
    CUDA_TRY(h, cudaMemcpyAsync(h->d_dt, &dt, sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return SPHGPU_OK;
}

sphgpu_status sphgpu_totals(sphgpu_handle* h, double out[9]) {
    return sphgpu_totals_frame(h, 0., out);
}

sphgpu_status sphgpu_totals_frame(sphgpu_handle* h, double omega, double out[9]) {
    if (!h || !out) {
        return SPHGPU_ERR_ARGUMENT;
    }
    if (!std::isfinite(omega)) {
        return fail(h, SPHGPU_ERR_ARGUMENT, "frame frequency must be finite");
    }
    launchTotals(h->s, omega, h->d_tot_partial, h->d_tot, h->stream);
    CUDA_TRY(h, cudaMemcpyAsync(out, h->d_tot, 9 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return SPHGPU_OK;
}

sphgpu_status sphgpu_check_finite(sphgpu_handle* h, uint64_t* first_bad) {
    if (!h) {
        return SPHGPU_ERR_ARGUMENT;
    }
    const unsigned long long none = ~0ull;
    CUDA_TRY(h, cudaMemcpyAsync(h->d_count, &none, sizeof(none), cudaMemcpyHostToDevice, h->stream));
    launchCheckFinite(h->s, h->d_count, h->stream);
    CUDA_TRY(h, cudaMemcpyAsync(h->h_pinned, h->d_count, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
        h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    const unsigned long long bad = h->h_pinned[0];
    if (first_bad) {
        *first_bad = bad;
    }
    if (bad != none) {
        return fail(h, SPHGPU_ERR_NONFINITE, "non-finite value at particle %llu", bad);
    }
    return SPHGPU_OK;
}

sphgpu_status sphgpu_set_profiling(sphgpu_handle* h, int32_t enabled) {
    if (!h) {
        return SPHGPU_ERR_ARGUMENT;
    }
    h->profiling = enabled != 0;
    return SPHGPU_OK;
}

sphgpu_status sphgpu_phase_times(sphgpu_handle* h, double out[SPHGPU_PHASE_COUNT], uint64_t* launches) {
    if (!h) {
        return SPHGPU_ERR_ARGUMENT;
    }
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    for (auto& m : h->marks) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, m.second.first, m.second.second);
        h->phase_ms[m.first] += ms;
        h->event_pool.push_back(m.second.first);
        h->event_pool.push_back(m.second.second);
    }
    h->marks.clear();
    if (out) {
        for (int k = 0; k < SPHGPU_PHASE_COUNT; ++k) {
            out[k] = h->phase_ms[k];
        }
    }
    if (launches) {
        *launches = h->launches;
    }
    for (int k = 0; k < SPHGPU_PHASE_COUNT; ++k) {
        h->phase_ms[k] = 0.;
    }
    h->launches = 0;
    return SPHGPU_OK;
}

sphgpu_status sphgpu_adjoint_forward(sphgpu_handle* h, const sphgpu_adjoint_config* cfg, double* loss) {
    if (!h || !cfg || !loss) {
        return SPHGPU_ERR_ARGUMENT;
    }
    if (requireSph(h) != SPHGPU_OK) {
        return SPHGPU_ERR_UNSUPPORTED;
    }
    if (cfg->rebuild_every == 0 || cfg->checkpoint_every == 0 || cfg->rebuild_every % cfg->checkpoint_every != 0) {
        return fail(h, SPHGPU_ERR_ARGUMENT,
            "adjoint: rebuild_every (%u) must be a positive multiple of checkpoint_every (%u)", cfg->rebuild_every,
            cfg->checkpoint_every);
    }
    if (!(cfg->dt > 0.) || !std::isfinite(cfg->dt) || !(cfg->gamma > 1.) || !std::isfinite(cfg->gamma) ||
        !std::isfinite(cfg->alpha) || !std::isfinite(cfg->beta)) {
        return fail(h, SPHGPU_ERR_ARGUMENT, "adjoint: dt must be positive, gamma above 1, alpha and beta finite");
    }
    if (cfg->precision != SPHGPU_PRECISION_FP64 && cfg->precision != SPHGPU_PRECISION_MIXED) {
        return fail(h, SPHGPU_ERR_ARGUMENT, "adjoint: unknown precision %d", cfg->precision);
    }
    cudaError_t e = adjointConfigure(h->adjoint, h->s.n, *cfg);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(h, SPHGPU_ERR_ALLOCATION, "adjoint: allocation failed: %s", cudaGetErrorString(e));
    }
    e = adjointForward(h->adjoint, h->s, h->grid, h->ph, h->d_lut_sph, h->d_lut_sph_f, loss, h->stream);
    h->launches += adjointTakeLaunches(h->adjoint);
    if (e != cudaSuccess) {
        return cudaFail(h, e, "adjoint forward");
    }
    return SPHGPU_OK;
}

sphgpu_status sphgpu_adjoint_backward(sphgpu_handle* h, double loss_bar, double* grad_r, double* grad_v,
    double* grad_rho, double* grad_u, double* grad_alpha) {
    if (!h) {
        return SPHGPU_ERR_ARGUMENT;
    }
    if (!adjointForwardDone(h->adjoint)) {
        return fail(h, SPHGPU_ERR_STATE, "adjoint: sphgpu_adjoint_forward has not run on this handle");
    }
    if (!std::isfinite(loss_bar)) {
        return fail(h, SPHGPU_ERR_ARGUMENT, "adjoint: loss_bar must be finite");
    }
    double alphaBar = 0.;
    cudaError_t e = adjointBackward(h->adjoint, h->s, h->grid, h->ph, h->d_lut_sph, h->d_lut_sph_f, loss_bar,
        &alphaBar, h->stream);
    if (e == cudaSuccess) {
        e = adjointGradients(h->adjoint, grad_r, grad_v, grad_rho, grad_u, h->stream);
    }
    h->launches += adjointTakeLaunches(h->adjoint);
    if (e != cudaSuccess) {
        return cudaFail(h, e, "adjoint backward");
    }
    if (grad_alpha) {
        *grad_alpha = alphaBar;
    }
    return SPHGPU_OK;
}

sphgpu_status sphgpu_collide(sphgpu_handle* h, double dt) {
    if (!h) {
        return SPHGPU_ERR_ARGUMENT;
    }
    if (!h->ph.nbody) {
        return fail(h, SPHGPU_ERR_UNSUPPORTED, "collide needs the N-body solver");
    }
    if (!(dt >= 0.)) {
        return fail(h, SPHGPU_ERR_ARGUMENT, "collide: dt must not be negative");
    }
    CUDA_TRY(h, cudaMemcpyAsync(h->d_dtc, &dt, sizeof(double), cudaMemcpyHostToDevice, h->stream));
    const sphgpu_status st = collideNbody(h, h->d_dtc, 1.);
    if (st != SPHGPU_OK) {
        return st;
    }
    CUDA_TRY(h, cudaGetLastError());
    return SPHGPU_OK;
}

sphgpu_status sphgpu_particle_count(sphgpu_handle* h, uint64_t* n) {
    if (!h || !n) {
        return SPHGPU_ERR_ARGUMENT;
    }
    *n = h->s.n;
    return SPHGPU_OK;
}

sphgpu_status sphgpu_collision_profile(sphgpu_handle* h, uint64_t out[4]) {
    if (!h || !out) {
        return SPHGPU_ERR_ARGUMENT;
    }
    for (int k = 0; k < 4; ++k) {
        out[k] = h->coll.profile[k];
    }
    return SPHGPU_OK;
}

sphgpu_status sphgpu_collision_stats(sphgpu_handle* h, uint64_t out[4]) {
    if (!h || !out) {
        return SPHGPU_ERR_ARGUMENT;
    }
    for (int k = 0; k < 4; ++k) {
        out[k] = h->coll.totals[k];
    }
    return SPHGPU_OK;
}

sphgpu_status sphgpu_get_time(sphgpu_handle* h, double* t) {
    if (!h || !t) {
        return SPHGPU_ERR_ARGUMENT;
    }
    CUDA_TRY(h, cudaMemcpyAsync(t, h->d_time, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return SPHGPU_OK;
}

sphgpu_status sphgpu_set_time(sphgpu_handle* h, double t) {
    if (!h) {
        return SPHGPU_ERR_ARGUMENT;
    }
    CUDA_TRY(h, cudaMemcpyAsync(h->d_time, &t, sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return SPHGPU_OK;
}

sphgpu_status sphgpu_take_removed(sphgpu_handle* h, uint32_t* removed, uint64_t capacity, uint64_t* count) {
    if (!h || !count || (capacity && !removed)) {
        return h ? fail(h, SPHGPU_ERR_ARGUMENT, "take_removed: NULL count or buffer") : SPHGPU_ERR_ARGUMENT;
    }
    if (!h->s.origin) {
        return fail(h, SPHGPU_ERR_UNSUPPORTED, "take_removed needs the N-body solver");
    }
    const uint32_t n = h->s.n;
    std::vector<uint32_t> origin(n);
    if (n) {
        CUDA_TRY(h, cudaMemcpyAsync(origin.data(), h->s.origin, n * sizeof(uint32_t), cudaMemcpyDeviceToHost,
            h->stream));
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    }
    std::vector<char> kept(h->n_sync, 0);
    for (uint32_t k : origin) {
        if (k < h->n_sync) {
            kept[k] = 1;
        }
    }
    uint64_t cnt = 0;
    for (uint32_t i = 0; i < h->n_sync; ++i) {
        if (!kept[i]) {
            if (cnt < capacity) {
                removed[cnt] = i;
            }
            ++cnt;
        }
    }
    *count = cnt;
    if (cnt > capacity) {
        return fail(h, SPHGPU_ERR_CAPACITY, "take_removed: %llu indices, room for %llu", (unsigned long long)cnt,
            (unsigned long long)capacity);
    }
    launchIota(h->s.origin, n, h->stream);
    CUDA_TRY(h, cudaGetLastError());
    h->n_sync = n;
    return SPHGPU_OK;
}

} // extern "C"
