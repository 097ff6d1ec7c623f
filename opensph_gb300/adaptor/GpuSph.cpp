/// \file GpuSph.cpp
/// \brief Reference-side adaptors over the libsphgpu C ABI (see GpuSph.h).

#include "GpuSph.h"
#include "timestepping/TimeStepCriterion.h"

#include "objects/Exceptions.h"
#include "sph/solvers/StandardSets.h"
#include "quantities/Attractor.h"
#include "quantities/IMaterial.h"
#include "quantities/Quantity.h"
#include "system/Statistics.h"
#include "thread/Scheduler.h"

#include <algorithm>
#include <string>

NAMESPACE_SPH_BEGIN

namespace Gpu {

namespace {

[[noreturn]] void raise(const bool setup, const std::string& msg) {
    if (setup) {
        throw InvalidSetup(String::fromAscii(msg.c_str()));
    }
    throw Exception(String::fromAscii(msg.c_str()));
}

// GravityKernelEnum (core/system/Settings.h:804-814) -> SPHGPU_GRAVITY_KERNEL_*
int gravityKernel(const RunSettings& settings) {
    switch (settings.get<GravityKernelEnum>(RunSettingsId::GRAVITY_KERNEL)) {
    case GravityKernelEnum::POINT_PARTICLES:
        return SPHGPU_GRAVITY_KERNEL_POINT_PARTICLES;
    case GravityKernelEnum::SOLID_SPHERES:
        return SPHGPU_GRAVITY_KERNEL_SOLID_SPHERES;
    default:
        return SPHGPU_GRAVITY_KERNEL_SPH_KERNEL;
    }
}

sphgpu_material toMaterial(const IMaterial& m) {
    sphgpu_material out{};
    const EosEnum eos = m.getParam<EosEnum>(BodySettingsId::EOS);
    if (eos == EosEnum::TILLOTSON) {
        out.eos = SPHGPU_EOS_TILLOTSON;
    } else if (eos == EosEnum::IDEAL_GAS) {
        out.eos = SPHGPU_EOS_IDEAL_GAS;
    } else {
        raise(true, "GPU path supports the Tillotson and ideal-gas equations of state");
    }
    const YieldingEnum yield = m.getParam<YieldingEnum>(BodySettingsId::RHEOLOGY_YIELDING);
    out.yielding = yield == YieldingEnum::VON_MISES ? SPHGPU_YIELDING_VON_MISES : SPHGPU_YIELDING_NONE;
    if (yield != YieldingEnum::VON_MISES && yield != YieldingEnum::NONE) {
        raise(true, "GPU path supports von Mises yielding only");
    }
    const FractureEnum frac = m.getParam<FractureEnum>(BodySettingsId::RHEOLOGY_DAMAGE);
    out.damage = frac == FractureEnum::SCALAR_GRADY_KIPP ? SPHGPU_DAMAGE_SCALAR_GRADY_KIPP : SPHGPU_DAMAGE_NONE;
    out.density = m.getParam<Float>(BodySettingsId::DENSITY);
    out.bulk_modulus = m.getParam<Float>(BodySettingsId::BULK_MODULUS);
    out.tillotson_nonlinear_b = m.getParam<Float>(BodySettingsId::TILLOTSON_NONLINEAR_B);
    out.tillotson_small_a = m.getParam<Float>(BodySettingsId::TILLOTSON_SMALL_A);
    out.tillotson_small_b = m.getParam<Float>(BodySettingsId::TILLOTSON_SMALL_B);
    out.tillotson_alpha = m.getParam<Float>(BodySettingsId::TILLOTSON_ALPHA);
    out.tillotson_beta = m.getParam<Float>(BodySettingsId::TILLOTSON_BETA);
    out.tillotson_sublimation = m.getParam<Float>(BodySettingsId::TILLOTSON_SUBLIMATION);
    out.tillotson_energy_iv = m.getParam<Float>(BodySettingsId::TILLOTSON_ENERGY_IV);
    out.tillotson_energy_cv = m.getParam<Float>(BodySettingsId::TILLOTSON_ENERGY_CV);
    out.adiabatic_index = m.getParam<Float>(BodySettingsId::ADIABATIC_INDEX);
    out.shear_modulus = m.getParam<Float>(BodySettingsId::SHEAR_MODULUS);
    out.elasticity_limit = m.getParam<Float>(BodySettingsId::ELASTICITY_LIMIT);
    out.melt_energy = m.getParam<Float>(BodySettingsId::MELT_ENERGY);
    out.young_modulus = m.getParam<Float>(BodySettingsId::YOUNG_MODULUS);
    const Interval rho = m.range(QuantityId::DENSITY);
    const Interval u = m.range(QuantityId::ENERGY);
    const Interval d = m.range(QuantityId::DAMAGE);
    out.density_range[0] = rho.lower();
    out.density_range[1] = rho.upper();
    out.energy_range[0] = u.lower();
    out.energy_range[1] = u.upper();
    out.damage_range[0] = d.lower();
    out.damage_range[1] = d.upper();
    out.density_min = m.minimal(QuantityId::DENSITY);
    out.energy_min = m.minimal(QuantityId::ENERGY);
    out.stress_min = m.minimal(QuantityId::DEVIATORIC_STRESS);
    out.damage_min = m.minimal(QuantityId::DAMAGE);
    return out;
}

template <typename T>
std::vector<double> packTensor(ArrayView<const T> a, int comps);

template <>
std::vector<double> packTensor(ArrayView<const TracelessTensor> a, int) {
    std::vector<double> out(5 * a.size());
    for (Size i = 0; i < a.size(); ++i) {
        out[5 * i + 0] = a[i](0, 0);
        out[5 * i + 1] = a[i](1, 1);
        out[5 * i + 2] = a[i](0, 1);
        out[5 * i + 3] = a[i](0, 2);
        out[5 * i + 4] = a[i](1, 2);
    }
    return out;
}

std::vector<uint32_t> packSize(ArrayView<const Size> a) {
    return std::vector<uint32_t>(a.begin(), a.end());
}

} // namespace

DeviceState::DeviceState(const RunSettings& settings, const Storage& storage, int precision) {
    for (Size k = 0; k < storage.getMaterialCnt(); ++k) {
        materials.push_back(toMaterial(storage.getMaterial(k).material()));
    }
    config = sphgpu_config{};
    config.particle_count = storage.getParticleCnt();
    config.material_count = uint32_t(materials.size());
    config.materials = materials.data();
    const Flags<ForceEnum> forces = settings.getFlags<ForceEnum>(RunSettingsId::SPH_SOLVER_FORCES);
    config.forces = (forces.has(ForceEnum::PRESSURE) ? SPHGPU_FORCE_PRESSURE : 0) |
                    (forces.has(ForceEnum::SOLID_STRESS) ? SPHGPU_FORCE_SOLID_STRESS : 0) |
                    (forces.has(ForceEnum::SELF_GRAVITY) ? SPHGPU_FORCE_SELF_GRAVITY : 0);
    config.adaptive_smoothing_length =
        settings.getFlags<SmoothingLengthEnum>(RunSettingsId::SPH_ADAPTIVE_SMOOTHING_LENGTH)
            .has(SmoothingLengthEnum::CONTINUITY_EQUATION);
    const Interval hRange = settings.get<Interval>(RunSettingsId::SPH_SMOOTHING_LENGTH_RANGE);
    config.smoothing_length_range[0] = hRange.lower();
    config.smoothing_length_range[1] = hRange.upper();
    config.av_alpha = settings.get<Float>(RunSettingsId::SPH_AV_ALPHA);
    config.av_beta = settings.get<Float>(RunSettingsId::SPH_AV_BETA);
    config.sum_only_undamaged = settings.get<bool>(RunSettingsId::SPH_SUM_ONLY_UNDAMAGED);
    config.gravity_multipole_order = settings.get<int>(RunSettingsId::GRAVITY_MULTIPOLE_ORDER);
    config.gravity_kernel = gravityKernel(settings);
    config.gravity_recomputation_period = settings.get<Float>(RunSettingsId::GRAVITY_RECOMPUTATION_PERIOD);
    config.gravity_constant = settings.get<Float>(RunSettingsId::GRAVITY_CONSTANT);
    config.gravity_opening_angle = settings.get<Float>(RunSettingsId::GRAVITY_OPENING_ANGLE);
    config.gravity_leaf_size = settings.get<int>(RunSettingsId::FINDER_LEAF_SIZE);
    config.integrator =
        settings.get<TimesteppingEnum>(RunSettingsId::TIMESTEPPING_INTEGRATOR) == TimesteppingEnum::LEAP_FROG
            ? SPHGPU_INTEGRATOR_LEAP_FROG
            : SPHGPU_INTEGRATOR_PREDICTOR_CORRECTOR;
    config.courant_number = settings.get<Float>(RunSettingsId::TIMESTEPPING_COURANT_NUMBER);
    config.max_timestep = settings.get<Float>(RunSettingsId::TIMESTEPPING_MAX_TIMESTEP);
    config.initial_timestep = settings.get<Float>(RunSettingsId::TIMESTEPPING_INITIAL_TIMESTEP);
    const Flags<TimeStepCriterionEnum> crit =
        settings.getFlags<TimeStepCriterionEnum>(RunSettingsId::TIMESTEPPING_CRITERION);
    config.timestep_criteria = (crit.has(TimeStepCriterionEnum::COURANT) ? SPHGPU_CRITERION_COURANT : 0) |
                               (crit.has(TimeStepCriterionEnum::DERIVATIVES) ? SPHGPU_CRITERION_DERIVATIVES : 0) |
                               (crit.has(TimeStepCriterionEnum::ACCELERATION) ? SPHGPU_CRITERION_ACCELERATION : 0) |
                               (crit.has(TimeStepCriterionEnum::DIVERGENCE) ? SPHGPU_CRITERION_DIVERGENCE : 0);
    config.derivative_factor = settings.get<Float>(RunSettingsId::TIMESTEPPING_DERIVATIVE_FACTOR);
    config.divergence_factor = settings.get<Float>(RunSettingsId::TIMESTEPPING_DIVERGENCE_FACTOR);
    config.max_change = settings.get<Float>(RunSettingsId::TIMESTEPPING_MAX_INCREASE);
    if (settings.get<Float>(RunSettingsId::TIMESTEPPING_MEAN_POWER) > -1.e3_f &&
        crit.has(TimeStepCriterionEnum::DERIVATIVES)) {
        raise(true, "GPU path implements the minimal-step derivative criterion only (timestep.mean_power = -inf)");
    }
    const SolverEnum solver = settings.get<SolverEnum>(RunSettingsId::SPH_SOLVER_TYPE);
    if (solver != SolverEnum::SYMMETRIC_SOLVER && solver != SolverEnum::ASYMMETRIC_SOLVER) {
        raise(true, "GPU path implements the symmetric and asymmetric solvers");
    }
    config.solver_type = solver == SolverEnum::ASYMMETRIC_SOLVER ? SPHGPU_SOLVER_ASYMMETRIC : SPHGPU_SOLVER_SYMMETRIC;
    config.correction_tensor = settings.get<bool>(RunSettingsId::SPH_STRAIN_RATE_CORRECTION_TENSOR) ? 1 : 0;
    config.precision = precision;
    config.device = 0;
    const int rc = sphgpu_create(&config, &handle);
    if (rc == SPHGPU_ERR_ARGUMENT || rc == SPHGPU_ERR_UNSUPPORTED) {
        raise(true, std::string("sphgpu: ") + sphgpu_last_error(nullptr));
    } else if (rc != SPHGPU_OK) {
        raise(false, std::string("sphgpu: ") + sphgpu_last_error(nullptr));
    }
}

DeviceState::~DeviceState() {
    sphgpu_destroy(handle);
}

void DeviceState::check(int status) const {
    if (status == SPHGPU_OK) {
        return;
    }
    const std::string msg = std::string("sphgpu: ") + sphgpu_last_error(handle);
    raise(status == SPHGPU_ERR_ARGUMENT || status == SPHGPU_ERR_UNSUPPORTED, msg);
}

void DeviceState::upload(const Storage& storage) {
    const Size n = storage.getParticleCnt();
    auto vec = [&](int order, ArrayView<const Vector> a) {
        // Vector is 4 contiguous doubles {x, y, z, h} (core/objects/geometry/Vector.h)
        check(sphgpu_set_quantity(handle, SPHGPU_Q_POSITION, order, &a[0][0], n));
    };
    ArrayView<const Vector> r, v, dv;
    tie(r, v, dv) = storage.getAll<Vector>(QuantityId::POSITION);
    vec(0, r);
    vec(1, v);
    vec(2, dv);
    check(sphgpu_set_quantity(handle, SPHGPU_Q_MASS, 0, &storage.getValue<Float>(QuantityId::MASS)[0], n));
    for (QuantityId id : { QuantityId::DENSITY, QuantityId::ENERGY }) {
        ArrayView<const Float> x, dx;
        tie(x, dx) = storage.getAll<Float>(id);
        check(sphgpu_set_quantity(handle, int(id), 0, &x[0], n));
        check(sphgpu_set_quantity(handle, int(id), 1, &dx[0], n));
    }
    const std::vector<uint32_t> flag = packSize(storage.getValue<Size>(QuantityId::FLAG));
    check(sphgpu_set_quantity(handle, SPHGPU_Q_FLAG, 0, flag.data(), n));
    std::vector<uint32_t> mat(n, 0);
    for (Size k = 0; k < storage.getMaterialCnt(); ++k) {
        for (Size i : storage.getMaterial(k).sequence()) {
            mat[i] = uint32_t(k);
        }
    }
    check(sphgpu_set_quantity(handle, SPHGPU_Q_MATERIAL_ID, 0, mat.data(), n));
    if (config.forces & SPHGPU_FORCE_SOLID_STRESS) {
        ArrayView<const TracelessTensor> S, dS;
        tie(S, dS) = storage.getAll<TracelessTensor>(QuantityId::DEVIATORIC_STRESS);
        const std::vector<double> s0 = packTensor(S, 5), s1 = packTensor(dS, 5);
        check(sphgpu_set_quantity(handle, SPHGPU_Q_DEVIATORIC_STRESS, 0, s0.data(), n));
        check(sphgpu_set_quantity(handle, SPHGPU_Q_DEVIATORIC_STRESS, 1, s1.data(), n));
        check(sphgpu_set_quantity(
            handle, SPHGPU_Q_STRESS_REDUCING, 0, &storage.getValue<Float>(QuantityId::STRESS_REDUCING)[0], n));
        if (storage.has(QuantityId::DAMAGE)) {
            ArrayView<const Float> D, dD;
            tie(D, dD) = storage.getAll<Float>(QuantityId::DAMAGE);
            check(sphgpu_set_quantity(handle, SPHGPU_Q_DAMAGE, 0, &D[0], n));
            check(sphgpu_set_quantity(handle, SPHGPU_Q_DAMAGE, 1, &dD[0], n));
            for (QuantityId id : { QuantityId::EPS_MIN, QuantityId::M_ZERO, QuantityId::EXPLICIT_GROWTH }) {
                check(sphgpu_set_quantity(handle, int(id), 0, &storage.getValue<Float>(id)[0], n));
            }
            const std::vector<uint32_t> nf = packSize(storage.getValue<Size>(QuantityId::N_FLAWS));
            check(sphgpu_set_quantity(handle, SPHGPU_Q_N_FLAWS, 0, nf.data(), n));
        }
    }
}

void DeviceState::download(Storage& storage, const bool derivativesOnly) const {
    const Size n = storage.getParticleCnt();
    ArrayView<Vector> r, v, dv;
    tie(r, v, dv) = storage.getAll<Vector>(QuantityId::POSITION);
    check(sphgpu_get_quantity(handle, SPHGPU_Q_POSITION, 2, &dv[0][0], n));
    // the finalize sets the smoothing-length derivative in the 4th component of v
    check(sphgpu_get_quantity(handle, SPHGPU_Q_POSITION, 1, &v[0][0], n));
    if (!derivativesOnly) {
        check(sphgpu_get_quantity(handle, SPHGPU_Q_POSITION, 0, &r[0][0], n));
    }
    for (QuantityId id : { QuantityId::DENSITY, QuantityId::ENERGY }) {
        ArrayView<Float> x, dx;
        tie(x, dx) = storage.getAll<Float>(id);
        check(sphgpu_get_quantity(handle, int(id), 1, &dx[0], n));
        if (!derivativesOnly) {
            check(sphgpu_get_quantity(handle, int(id), 0, &x[0], n));
        }
    }
    check(sphgpu_get_quantity(handle, SPHGPU_Q_PRESSURE, 0, &storage.getValue<Float>(QuantityId::PRESSURE)[0], n));
    check(sphgpu_get_quantity(
        handle, SPHGPU_Q_SOUND_SPEED, 0, &storage.getValue<Float>(QuantityId::SOUND_SPEED)[0], n));
    if (storage.has(QuantityId::VELOCITY_DIVERGENCE)) {
        check(sphgpu_get_quantity(handle,
            SPHGPU_Q_VELOCITY_DIVERGENCE,
            0,
            &storage.getValue<Float>(QuantityId::VELOCITY_DIVERGENCE)[0],
            n));
    }
    {
        std::vector<uint32_t> cnt(n);
        check(sphgpu_get_quantity(handle, SPHGPU_Q_NEIGHBOR_CNT, 0, cnt.data(), n));
        ArrayView<Size> nc = storage.getValue<Size>(QuantityId::NEIGHBOR_CNT);
        std::copy(cnt.begin(), cnt.end(), nc.begin());
    }
    if (config.forces & SPHGPU_FORCE_SOLID_STRESS) {
        std::vector<double> s(5 * n), g(6 * n);
        ArrayView<TracelessTensor> S, dS;
        tie(S, dS) = storage.getAll<TracelessTensor>(QuantityId::DEVIATORIC_STRESS);
        for (int order = 0; order < 2; ++order) {
            if (order == 0 && derivativesOnly) {
                // von Mises reduces S in place during the evaluation: S is an output as well
            }
            check(sphgpu_get_quantity(handle, SPHGPU_Q_DEVIATORIC_STRESS, order, s.data(), n));
            ArrayView<TracelessTensor> dst = order == 0 ? S : dS;
            for (Size i = 0; i < n; ++i) {
                dst[i] = TracelessTensor(s[5 * i], s[5 * i + 1], s[5 * i + 2], s[5 * i + 3], s[5 * i + 4]);
            }
        }
        check(sphgpu_get_quantity(handle, SPHGPU_Q_VELOCITY_GRADIENT, 0, g.data(), n));
        ArrayView<SymmetricTensor> gv = storage.getValue<SymmetricTensor>(QuantityId::VELOCITY_GRADIENT);
        for (Size i = 0; i < n; ++i) {
            gv[i] = SymmetricTensor(
                Vector(g[6 * i], g[6 * i + 1], g[6 * i + 2]), Vector(g[6 * i + 3], g[6 * i + 4], g[6 * i + 5]));
        }
        check(sphgpu_get_quantity(
            handle, SPHGPU_Q_STRESS_REDUCING, 0, &storage.getValue<Float>(QuantityId::STRESS_REDUCING)[0], n));
        if (storage.has(QuantityId::DAMAGE)) {
            ArrayView<Float> D, dD;
            tie(D, dD) = storage.getAll<Float>(QuantityId::DAMAGE);
            check(sphgpu_get_quantity(handle, SPHGPU_Q_DAMAGE, 1, &dD[0], n));
            if (!derivativesOnly) {
                check(sphgpu_get_quantity(handle, SPHGPU_Q_DAMAGE, 0, &D[0], n));
            }
        }
    }
}

// ---------------------------------------------------------------------------------------------------------

GpuSolver::GpuSolver(IScheduler& UNUSED(scheduler), const RunSettings& settings, const int precision)
    : settings(settings)
    , precision(precision) {}

GpuSolver::~GpuSolver() = default;

DeviceState& GpuSolver::getDevice(const Storage& storage) const {
    if (!device || device->particleCount() != storage.getParticleCnt()) {
        device = std::make_unique<DeviceState>(settings, storage, precision);
    }
    return *device;
}

void GpuSolver::integrate(Storage& storage, Statistics& stats) {
    DeviceState& dev = this->getDevice(storage);
    dev.upload(storage);
    dev.check(sphgpu_integrate(dev.get()));
    dev.download(storage, true);
    double times[SPHGPU_PHASE_COUNT];
    uint64_t launches = 0;
    if (sphgpu_phase_times(dev.get(), times, &launches) == SPHGPU_OK) {
        stats.set(StatisticsId::GRAVITY_BUILD_TIME, int(times[SPHGPU_PHASE_GRAVITY_BUILD]));
        stats.set(StatisticsId::GRAVITY_EVAL_TIME, int(times[SPHGPU_PHASE_GRAVITY_EVAL]));
        stats.set(StatisticsId::SPH_EVAL_TIME, int(times[SPHGPU_PHASE_SPH_EVAL] + times[SPHGPU_PHASE_NEIGHBORS]));
    }
}

void GpuSolver::create(Storage& storage, IMaterial& material) const {
    // same quantities as the reference solver: the standard equation set creates them
    // (SymmetricSolver::create, core/sph/solvers/SymmetricSolver.cpp:97-104)
    storage.insert<Size>(QuantityId::NEIGHBOR_CNT, OrderEnum::ZERO, 0);
    getStandardEquations(settings).create(storage, material);
}

namespace {

/// The time step computed by the device at the end of its step (the criteria of the settings, evaluated by
/// sphgpu_step); replaces the host-side MultiCriterion so that ITimeStepping::step reads no host quantity.
class GpuCriterion : public ITimeStepCriterion {
    std::shared_ptr<GpuTimeStepping::Link> link;
    Float initial;

public:
    GpuCriterion(std::shared_ptr<GpuTimeStepping::Link> link, const Float initial)
        : link(std::move(link))
        , initial(initial) {}

    virtual TimeStep compute(IScheduler& UNUSED(scheduler),
        Storage& UNUSED(storage),
        const Float maxStep,
        Statistics& UNUSED(stats),
        ArrayView<TimeStep> UNUSED(dts)) override {
        if (!link->device) {
            return { initial, CriterionId::INITIAL_VALUE };
        }
        double dt = 0.;
        link->device->check(sphgpu_get_timestep(link->device->get(), &dt));
        return { Float(dt), dt >= maxStep ? CriterionId::MAXIMAL_VALUE : CriterionId::CFL_CONDITION };
    }
};

} // namespace

GpuTimeStepping::GpuTimeStepping(const SharedPtr<Storage>& storage, const RunSettings& settings, const SyncMode mode)
    : ITimeStepping(storage,
          settings,
          makeAuto<GpuCriterion>(std::make_shared<Link>(), settings.get<Float>(RunSettingsId::TIMESTEPPING_INITIAL_TIMESTEP)))
    , mode(mode) {
    // the criterion constructed above owns the first Link; share it
    link = std::make_shared<Link>();
    criterion = makeAuto<GpuCriterion>(link, settings.get<Float>(RunSettingsId::TIMESTEPPING_INITIAL_TIMESTEP));
    storage->zeroHighestDerivatives(SEQUENTIAL);
}

void GpuTimeStepping::stepParticles(IScheduler& UNUSED(scheduler), ISolver& solver, Statistics& UNUSED(stats)) {
    GpuSolver* gpu = dynamic_cast<GpuSolver*>(&solver);
    if (!gpu) {
        raise(true, "GpuTimeStepping requires GpuSolver");
    }
    DeviceState& dev = gpu->getDevice(*storage);
    if (link->device != &dev) {
        link->device = &dev;
        uploaded = false;
    }
    if (mode == SyncMode::EVERY_STEP || !uploaded) {
        dev.upload(*storage);
        uploaded = true;
    }
    dev.check(sphgpu_set_timestep(dev.get(), timeStep));
    dev.check(sphgpu_step(dev.get(), 1));
    hostCurrent = false;
    if (mode == SyncMode::EVERY_STEP) {
        this->sync();
    }
}

void GpuTimeStepping::sync() {
    if (hostCurrent || !link->device) {
        return;
    }
    link->device->download(*storage, false);
    hostCurrent = true;
    syncs++;
}

void GpuTimeStepping::invalidate() {
    uploaded = false;
    hostCurrent = true;
}

GpuOutput::GpuOutput(AutoPtr<IOutput>&& output, GpuTimeStepping& stepping)
    : IOutput(OutputFile())
    , output(std::move(output))
    , stepping(stepping) {}

Expected<Path> GpuOutput::dump(const Storage& storage, const Statistics& stats) {
    stepping.sync();
    return output->dump(storage, stats);
}

// ---------------------------------------------------------------------------------------------------------

GpuBarnesHut::GpuBarnesHut(const RunSettings& settings)
    : settings(settings) {}

GpuBarnesHut::~GpuBarnesHut() = default;

void GpuBarnesHut::build(IScheduler& UNUSED(scheduler), const Storage& storage) {
    if (!device || device->particleCount() != storage.getParticleCnt()) {
        device = std::make_unique<DeviceState>(settings, storage, SPHGPU_PRECISION_FP64);
    }
    const Size n = storage.getParticleCnt();
    positions = storage.getValue<Vector>(QuantityId::POSITION);
    finderCurrent = false;
    device->check(
        sphgpu_set_quantity(device->get(), SPHGPU_Q_POSITION, 0, &storage.getValue<Vector>(QuantityId::POSITION)[0][0], n));
    device->check(sphgpu_set_quantity(device->get(), SPHGPU_Q_MASS, 0, &storage.getValue<Float>(QuantityId::MASS)[0], n));
    device->check(sphgpu_gravity_build(device->get()));
}

void GpuBarnesHut::evalSelfGravity(IScheduler& UNUSED(scheduler), ArrayView<Vector> dv, Statistics& stats) const {
    device->check(sphgpu_gravity_eval(device->get(), &dv[0][0], dv.size()));
    uint64_t s[3];
    device->check(sphgpu_gravity_stats(device->get(), s));
    stats.set<int>(StatisticsId::GRAVITY_NODES_APPROX, int(s[0]));
    stats.set<int>(StatisticsId::GRAVITY_NODES_EXACT, int(s[1]));
    stats.set<int>(StatisticsId::GRAVITY_NODE_COUNT, int(s[2]));
}

void GpuBarnesHut::evalAttractors(IScheduler& UNUSED(scheduler),
    ArrayView<Attractor> attractors,
    ArrayView<Vector> dv) const {
    if (attractors.empty()) {
        return;
    }
    // BarnesHut::evalAttractors (core/gravity/BarnesHut.cpp:100-125) on the device
    std::vector<double> att, acc;
    for (const Attractor& a : attractors) {
        att.insert(att.end(), { a.position[X], a.position[Y], a.position[Z], a.radius, a.mass });
        acc.insert(acc.end(), { a.acceleration[X], a.acceleration[Y], a.acceleration[Z] });
    }
    device->check(sphgpu_gravity_attractors(device->get(), att.data(), attractors.size(), acc.data(),
        dv.empty() ? nullptr : &dv[0][0], dv.size()));
    for (Size k = 0; k < attractors.size(); ++k) {
        Vector& out = attractors[k].acceleration;
        out = Vector(acc[3 * k], acc[3 * k + 1], acc[3 * k + 2], out[H]);
    }
}

Vector GpuBarnesHut::evalAcceleration(const Vector& r0) const {
    double p[4] = { r0[X], r0[Y], r0[Z], r0[H] }, a[4];
    device->check(sphgpu_gravity_eval_points(device->get(), p, 1, a));
    return Vector(a[0], a[1], a[2]);
}

Float GpuBarnesHut::evalEnergy(IScheduler& UNUSED(scheduler), Statistics& UNUSED(stats)) const {
    NOT_IMPLEMENTED; // as the reference BarnesHut (core/gravity/BarnesHut.cpp:114-116)
}

RawPtr<const IBasicFinder> GpuBarnesHut::getFinder() const {
    if (!finderCurrent) {
        if (!finder) {
            finder = std::make_unique<GpuFinder>(settings);
        }
        finder->build(SEQUENTIAL, positions);
        finderCurrent = true;
    }
    return finder.get();
}

// ---------------------------------------------------------------------------------------------------------

GpuFinder::GpuFinder(const RunSettings& UNUSED(settings)) {}

GpuFinder::~GpuFinder() {
    sphgpu_destroy(handle);
}

void GpuFinder::buildImpl(IScheduler& UNUSED(scheduler), ArrayView<const Vector> points) {
    const Size n = points.size();
    if (!handle || handleCount != n) {
        sphgpu_destroy(handle);
        handle = nullptr;
        sphgpu_material mat{};
        mat.eos = SPHGPU_EOS_IDEAL_GAS;
        mat.density = 1.;
        mat.adiabatic_index = 1.4;
        sphgpu_config cfg{};
        cfg.particle_count = n;
        cfg.material_count = 1;
        cfg.materials = &mat;
        cfg.forces = SPHGPU_FORCE_PRESSURE;
        cfg.gravity_leaf_size = 25;
        cfg.gravity_multipole_order = 3;
        if (sphgpu_create(&cfg, &handle) != SPHGPU_OK) {
            handle = nullptr;
            raise(false, std::string("sphgpu: ") + sphgpu_last_error(nullptr));
        }
        handleCount = n;
    }
    auto check = [&](int rc) {
        if (rc != SPHGPU_OK) {
            raise(false, std::string("sphgpu: ") + sphgpu_last_error(handle));
        }
    };
    start.assign(n + 1, 0);
    neighbours.clear();
    if (n == 0) {
        return;
    }
    check(sphgpu_set_quantity(handle, SPHGPU_Q_POSITION, 0, &points[0][0], n));
    // the ball of radius 2 h_i of every particle, directed pairs sorted by i then j
    uint64_t npairs = 0;
    const int rc = sphgpu_get_radius_pairs(handle, nullptr, nullptr, 0, &npairs);
    if (rc != SPHGPU_OK && rc != SPHGPU_ERR_CAPACITY) {
        check(rc);
    }
    std::vector<uint32_t> pi(npairs), pj(npairs);
    if (npairs) {
        check(sphgpu_get_radius_pairs(handle, pi.data(), pj.data(), npairs, &npairs));
    }
    for (uint64_t k = 0; k < npairs; ++k) {
        start[pi[k] + 1]++;
    }
    for (Size i = 0; i < n; ++i) {
        start[i + 1] += start[i];
    }
    neighbours.assign(pj.begin(), pj.end());
}

template <bool FindAll>
Size GpuFinder::find(const Vector& pos, const Size index, const Float radius, Array<NeighborRecord>& neighs) const {
    if (index < values.size() && radius == 2._f * values[index][H]) {
        // the query of the SPH loops, from the lists of the build
        for (Size k = start[index]; k < start[index + 1]; ++k) {
            const Size j = neighbours[k];
            if (FindAll || rank[j] < rank[index]) {
                neighs.push(NeighborRecord{ j, getSqrLength(values[j] - pos) });
            }
        }
        if (FindAll) {
            neighs.push(NeighborRecord{ index, 0._f });
        }
        return neighs.size();
    }
    // any other ball on the device
    const double p[3] = { pos[X], pos[Y], pos[Z] };
    uint64_t count = 0;
    if (queryIdx.empty()) {
        queryIdx.resize(256);
        queryDistSqr.resize(256);
    }
    int rc = sphgpu_find_neighbors(handle, p, radius, queryIdx.data(), queryDistSqr.data(), queryIdx.size(), &count);
    if (rc == SPHGPU_ERR_CAPACITY) {
        queryIdx.resize(count);
        queryDistSqr.resize(count);
        rc = sphgpu_find_neighbors(handle, p, radius, queryIdx.data(), queryDistSqr.data(), queryIdx.size(), &count);
    }
    if (rc != SPHGPU_OK) {
        raise(false, std::string("sphgpu: ") + sphgpu_last_error(handle));
    }
    for (uint64_t k = 0; k < count; ++k) {
        const Size j = queryIdx[k];
        if (FindAll || index >= values.size() || rank[j] < rank[index]) {
            neighs.push(NeighborRecord{ j, queryDistSqr[k] });
        }
    }
    return neighs.size();
}

template Size GpuFinder::find<true>(const Vector&, const Size, const Float, Array<NeighborRecord>&) const;
template Size GpuFinder::find<false>(const Vector&, const Size, const Float, Array<NeighborRecord>&) const;

} // namespace Gpu

NAMESPACE_SPH_END

NAMESPACE_SPH_BEGIN

namespace Gpu {

GpuHardSphereSolver::GpuHardSphereSolver(IScheduler& UNUSED(scheduler), const RunSettings& settings, int precision)
    : settings(settings)
    , precision(precision) {
    if (settings.get<bool>(RunSettingsId::NBODY_INERTIA_TENSOR)) {
        raise(true, "GPU N-body solver: the inertia tensor of particles is not implemented");
    }
}

GpuHardSphereSolver::~GpuHardSphereSolver() {
    sphgpu_destroy(handle);
}

void GpuHardSphereSolver::check(int status) const {
    if (status == SPHGPU_OK) {
        return;
    }
    const std::string msg = std::string("sphgpu: ") + sphgpu_last_error(handle);
    raise(status == SPHGPU_ERR_ARGUMENT || status == SPHGPU_ERR_UNSUPPORTED, msg);
}

void GpuHardSphereSolver::ensure(const Storage& storage) {
    if (handle && count == storage.getParticleCnt()) {
        return;
    }
    sphgpu_destroy(handle);
    handle = nullptr;
    sphgpu_config config{};
    config.particle_count = storage.getParticleCnt();
    config.solver_type = SPHGPU_SOLVER_NBODY_HARD_SPHERE;
    config.integrator = SPHGPU_INTEGRATOR_LEAP_FROG;
    config.forces = SPHGPU_FORCE_SELF_GRAVITY;
    config.gravity_kernel = gravityKernel(settings);
    config.gravity_multipole_order = settings.get<int>(RunSettingsId::GRAVITY_MULTIPOLE_ORDER);
    config.gravity_constant = settings.get<Float>(RunSettingsId::GRAVITY_CONSTANT);
    config.gravity_opening_angle = settings.get<Float>(RunSettingsId::GRAVITY_OPENING_ANGLE);
    config.gravity_leaf_size = settings.get<int>(RunSettingsId::FINDER_LEAF_SIZE);
    config.gravity_recomputation_period = settings.get<Float>(RunSettingsId::GRAVITY_RECOMPUTATION_PERIOD);
    config.max_timestep = settings.get<Float>(RunSettingsId::TIMESTEPPING_MAX_TIMESTEP);
    config.initial_timestep = settings.get<Float>(RunSettingsId::TIMESTEPPING_INITIAL_TIMESTEP);
    config.derivative_factor = settings.get<Float>(RunSettingsId::TIMESTEPPING_DERIVATIVE_FACTOR);
    config.max_change = settings.get<Float>(RunSettingsId::TIMESTEPPING_MAX_INCREASE);
    // Factory::getCollisionHandler / getOverlapHandler (core/system/Factory.cpp:415-450)
    switch (settings.get<CollisionHandlerEnum>(RunSettingsId::COLLISION_HANDLER)) {
    case CollisionHandlerEnum::NONE:
        config.collision_handler = SPHGPU_COLLISION_NONE;
        break;
    case CollisionHandlerEnum::PERFECT_MERGING:
        config.collision_handler = SPHGPU_COLLISION_PERFECT_MERGING;
        break;
    case CollisionHandlerEnum::ELASTIC_BOUNCE:
        config.collision_handler = SPHGPU_COLLISION_ELASTIC_BOUNCE;
        break;
    default:
        config.collision_handler = SPHGPU_COLLISION_MERGE_OR_BOUNCE;
        break;
    }
    config.overlap_handler = int32_t(settings.get<OverlapEnum>(RunSettingsId::COLLISION_OVERLAP));
    config.restitution_normal = settings.get<Float>(RunSettingsId::COLLISION_RESTITUTION_NORMAL);
    config.restitution_tangent = settings.get<Float>(RunSettingsId::COLLISION_RESTITUTION_TANGENT);
    config.allowed_overlap = settings.get<Float>(RunSettingsId::COLLISION_ALLOWED_OVERLAP);
    config.bounce_merge_limit = settings.get<Float>(RunSettingsId::COLLISION_BOUNCE_MERGE_LIMIT);
    config.rotation_merge_limit = settings.get<Float>(RunSettingsId::COLLISION_ROTATION_MERGE_LIMIT);
    config.max_bounces = uint32_t(settings.get<int>(RunSettingsId::COLLISION_MAX_BOUNCES));
    config.precision = precision;
    const int rc = sphgpu_create(&config, &handle);
    if (rc != SPHGPU_OK) {
        raise(rc == SPHGPU_ERR_ARGUMENT || rc == SPHGPU_ERR_UNSUPPORTED,
            std::string("sphgpu: ") + sphgpu_last_error(nullptr));
    }
    count = config.particle_count;
}

void GpuHardSphereSolver::upload(const Storage& storage) {
    const Size n = storage.getParticleCnt();
    ArrayView<const Vector> r, v, dv;
    tie(r, v, dv) = storage.getAll<Vector>(QuantityId::POSITION);
    check(sphgpu_set_quantity(handle, SPHGPU_Q_POSITION, 0, &r[0][0], n));
    check(sphgpu_set_quantity(handle, SPHGPU_Q_POSITION, 1, &v[0][0], n));
    check(sphgpu_set_quantity(handle, SPHGPU_Q_MASS, 0, &storage.getValue<Float>(QuantityId::MASS)[0], n));
    check(sphgpu_set_quantity(
        handle, SPHGPU_Q_ANGULAR_FREQUENCY, 0, &storage.getValue<Vector>(QuantityId::ANGULAR_FREQUENCY)[0][0], n));
}

void GpuHardSphereSolver::download(Storage& storage, bool positions) {
    const Size n = storage.getParticleCnt();
    ArrayView<Vector> r, v, dv;
    tie(r, v, dv) = storage.getAll<Vector>(QuantityId::POSITION);
    check(sphgpu_get_quantity(handle, SPHGPU_Q_POSITION, 1, &v[0][0], n));
    check(sphgpu_get_quantity(handle, SPHGPU_Q_POSITION, 2, &dv[0][0], n));
    if (positions) {
        check(sphgpu_get_quantity(handle, SPHGPU_Q_POSITION, 0, &r[0][0], n));
        check(sphgpu_get_quantity(handle, SPHGPU_Q_MASS, 0, &storage.getValue<Float>(QuantityId::MASS)[0], n));
        check(sphgpu_get_quantity(
            handle, SPHGPU_Q_ANGULAR_FREQUENCY, 0, &storage.getValue<Vector>(QuantityId::ANGULAR_FREQUENCY)[0][0], n));
    }
}

void GpuHardSphereSolver::integrate(Storage& storage, Statistics& stats) {
    if (storage.getParticleCnt() == 0) {
        return;
    }
    ensure(storage);
    upload(storage);
    check(sphgpu_integrate(handle));
    download(storage, false);
    double times[SPHGPU_PHASE_COUNT];
    if (sphgpu_phase_times(handle, times, nullptr) == SPHGPU_OK) {
        stats.set(StatisticsId::GRAVITY_EVAL_TIME, int(times[SPHGPU_PHASE_GRAVITY_BUILD] + times[SPHGPU_PHASE_GRAVITY_EVAL]));
    }
}

void GpuHardSphereSolver::collide(Storage& storage, Statistics& stats, const Float dt) {
    if (settings.get<CollisionHandlerEnum>(RunSettingsId::COLLISION_HANDLER) == CollisionHandlerEnum::NONE ||
        storage.getParticleCnt() == 0) {
        return; // HardSphereSolver::collide ignores all collisions without a handler
    }
    ensure(storage);
    upload(storage);
    check(sphgpu_collide(handle, dt));
    // the particles merged away, as the argument of Storage::remove (NBodySolver.cpp:478-481)
    uint64_t removedCount = 0;
    std::vector<uint32_t> removed(storage.getParticleCnt());
    check(sphgpu_take_removed(handle, removed.data(), removed.size(), &removedCount));
    if (removedCount > 0) {
        Array<Size> idxs(removedCount);
        for (uint64_t k = 0; k < removedCount; ++k) {
            idxs[k] = removed[k];
        }
        storage.remove(idxs, Storage::IndicesFlag::INDICES_SORTED | Storage::IndicesFlag::PROPAGATE);
        count = storage.getParticleCnt();
    }
    download(storage, true);
    // CollisionStats (NBodySolver.cpp:119-163): the counts of this call
    uint64_t totals[4];
    check(sphgpu_collision_stats(handle, totals));
    stats.set(StatisticsId::TOTAL_COLLISION_COUNT, int(totals[0] - collisionTotals[0]));
    stats.set(StatisticsId::MERGER_COUNT, int(totals[1] - collisionTotals[1]));
    stats.set(StatisticsId::BOUNCE_COUNT, int(totals[2] - collisionTotals[2]));
    stats.set(StatisticsId::OVERLAP_COUNT, int(totals[3] - collisionTotals[3]));
    for (int k = 0; k < 4; ++k) {
        collisionTotals[k] = totals[k];
    }
}

void GpuHardSphereSolver::create(Storage& storage, IMaterial& UNUSED(material)) const {
    // HardSphereSolver::create without the inertia tensor (core/gravity/NBodySolver.cpp:487-507)
    storage.insert<Vector>(QuantityId::ANGULAR_FREQUENCY, OrderEnum::ZERO, Vector(0._f));
}

} // namespace Gpu

NAMESPACE_SPH_END
