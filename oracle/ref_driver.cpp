// Golden-vector generator built against the REFERENCE OpenSPH core library (test infrastructure only).
//
// This program is compiled from the reference's own core/*.cpp sources by `make -C oracle ref` and run by
// tests/golden/make_golden.py in the build container, where the reference tree exists. It drives the
// reference through its public library entry (InitialConditions -> Factory::getSolver -> solver.create ->
// Factory::getTimeStepping -> ITimeStepping::step, exactly the entry used by the reference's own solver
// tests and examples, core/sph/solvers/test/Solvers.cpp:42-121, examples/01_hello_asteroid) with the
// SEQUENTIAL scheduler (run.thread.cnt = 1), and writes every quantity of the hot path to a flat binary
// file that make_golden.py converts into tests/golden/*.npz fixtures.
//
// Output format: a sequence of records "<name> <dtype> <count>\n" followed by count raw elements.

#include "Sph.h"
#include "gravity/BarnesHut.h"
#include "gravity/BruteForceGravity.h"
#include "gravity/Moments.h"
#include "gravity/NBodySolver.h"
#include "physics/Integrals.h"
#include "quantities/Attractor.h"
#include "objects/finders/KdTree.h"
#include "sph/kernel/GravityKernel.h"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <string>
#include <vector>

using namespace Sph;

namespace {

struct Writer {
    FILE* f = nullptr;
    explicit Writer(const char* path) {
        f = std::fopen(path, "wb");
        if (!f) {
            std::fprintf(stderr, "cannot open %s\n", path);
            std::exit(2);
        }
    }
    ~Writer() {
        std::fclose(f);
    }
    void f64(const std::string& name, const std::vector<double>& v) {
        std::fprintf(f, "%s f8 %zu\n", name.c_str(), v.size());
        std::fwrite(v.data(), sizeof(double), v.size(), f);
    }
    void u32(const std::string& name, const std::vector<uint32_t>& v) {
        std::fprintf(f, "%s u4 %zu\n", name.c_str(), v.size());
        std::fwrite(v.data(), sizeof(uint32_t), v.size(), f);
    }
    void scalar(const std::string& name, double x) {
        f64(name, std::vector<double>{ x });
    }
};

// splitmix64 counter RNG + Box-Muller: the seeded velocity field of the harness. The generated values are
// written to the fixture, so consumers never need to regenerate them.
struct SplitMix {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uniform() {
        return (double(next() >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    }
    double normal() {
        const double u1 = uniform(), u2 = uniform();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * 3.14159265358979323846 * u2);
    }
};

std::vector<double> vec4(ArrayView<const Vector> a) {
    std::vector<double> out(4 * a.size());
    for (Size i = 0; i < a.size(); ++i) {
        for (int k = 0; k < 4; ++k) {
            out[4 * i + k] = a[i][k];
        }
    }
    return out;
}

std::vector<double> flt(ArrayView<const Float> a) {
    return std::vector<double>(a.begin(), a.end());
}

std::vector<uint32_t> sz(ArrayView<const Size> a) {
    return std::vector<uint32_t>(a.begin(), a.end());
}

std::vector<double> traceless(ArrayView<const TracelessTensor> a) {
    // independent components xx, yy, xy, xz, yz
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

std::vector<double> symmetric(ArrayView<const SymmetricTensor> a) {
    // xx, yy, zz, xy, xz, yz
    std::vector<double> out(6 * a.size());
    for (Size i = 0; i < a.size(); ++i) {
        out[6 * i + 0] = a[i](0, 0);
        out[6 * i + 1] = a[i](1, 1);
        out[6 * i + 2] = a[i](2, 2);
        out[6 * i + 3] = a[i](0, 1);
        out[6 * i + 4] = a[i](0, 2);
        out[6 * i + 5] = a[i](1, 2);
    }
    return out;
}

void dumpState(Writer& w, const std::string& pre, Storage& s) {
    ArrayView<const Vector> r, v, dv;
    tie(r, v, dv) = s.getAll<Vector>(QuantityId::POSITION);
    w.f64(pre + "r", vec4(r));
    w.f64(pre + "v", vec4(v));
    w.f64(pre + "dv", vec4(dv));
    w.f64(pre + "m", flt(s.getValue<Float>(QuantityId::MASS)));
    {
        ArrayView<const Float> rho, drho;
        tie(rho, drho) = s.getAll<Float>(QuantityId::DENSITY);
        w.f64(pre + "rho", flt(rho));
        w.f64(pre + "drho", flt(drho));
    }
    {
        ArrayView<const Float> u, du;
        tie(u, du) = s.getAll<Float>(QuantityId::ENERGY);
        w.f64(pre + "u", flt(u));
        w.f64(pre + "du", flt(du));
    }
    w.f64(pre + "p", flt(s.getValue<Float>(QuantityId::PRESSURE)));
    w.f64(pre + "cs", flt(s.getValue<Float>(QuantityId::SOUND_SPEED)));
    if (s.has(QuantityId::VELOCITY_DIVERGENCE)) {
        w.f64(pre + "divv", flt(s.getValue<Float>(QuantityId::VELOCITY_DIVERGENCE)));
    }
    if (s.has(QuantityId::NEIGHBOR_CNT)) {
        w.u32(pre + "ncnt", sz(s.getValue<Size>(QuantityId::NEIGHBOR_CNT)));
    }
    w.u32(pre + "flag", sz(s.getValue<Size>(QuantityId::FLAG)));
    if (s.has(QuantityId::DEVIATORIC_STRESS)) {
        ArrayView<const TracelessTensor> S, dS;
        tie(S, dS) = s.getAll<TracelessTensor>(QuantityId::DEVIATORIC_STRESS);
        w.f64(pre + "S", traceless(S));
        w.f64(pre + "dS", traceless(dS));
    }
    if (s.has(QuantityId::VELOCITY_GRADIENT)) {
        w.f64(pre + "gradv", symmetric(s.getValue<SymmetricTensor>(QuantityId::VELOCITY_GRADIENT)));
    }
    if (s.has(QuantityId::STRAIN_RATE_CORRECTION_TENSOR)) {
        w.f64(pre + "corr", symmetric(s.getValue<SymmetricTensor>(QuantityId::STRAIN_RATE_CORRECTION_TENSOR)));
    }
    if (s.has(QuantityId::DAMAGE)) {
        ArrayView<const Float> D, dD;
        tie(D, dD) = s.getAll<Float>(QuantityId::DAMAGE);
        w.f64(pre + "D", flt(D));
        w.f64(pre + "dD", flt(dD));
        w.f64(pre + "eps_min", flt(s.getValue<Float>(QuantityId::EPS_MIN)));
        w.f64(pre + "m_zero", flt(s.getValue<Float>(QuantityId::M_ZERO)));
        w.f64(pre + "growth", flt(s.getValue<Float>(QuantityId::EXPLICIT_GROWTH)));
        w.u32(pre + "n_flaws", sz(s.getValue<Size>(QuantityId::N_FLAWS)));
    }
    if (s.has(QuantityId::STRESS_REDUCING)) {
        w.f64(pre + "reduce", flt(s.getValue<Float>(QuantityId::STRESS_REDUCING)));
    }
}

void dumpMaterials(Writer& w, Storage& s) {
    // per-particle material index and, per material, the clamping ranges and the parameters the hot path
    // needs (YOUNG_MODULUS is derived by ScalarGradyKippModel::setFlaws, so it must be read back here).
    std::vector<uint32_t> mat(s.getParticleCnt(), 0);
    std::vector<double> ranges;
    std::vector<double> young;
    std::vector<double> minimals;
    for (Size k = 0; k < s.getMaterialCnt(); ++k) {
        MaterialView mv = s.getMaterial(k);
        for (Size i : mv.sequence()) {
            mat[i] = uint32_t(k);
        }
        for (QuantityId id : { QuantityId::DENSITY, QuantityId::ENERGY, QuantityId::DAMAGE }) {
            const Interval range = mv->range(id);
            ranges.push_back(range.lower());
            ranges.push_back(range.upper());
        }
        young.push_back(mv->getParam<Float>(BodySettingsId::YOUNG_MODULUS));
        // IMaterial::minimal of the first-order quantities (DerivativeCriterion)
        for (QuantityId id :
            { QuantityId::DENSITY, QuantityId::ENERGY, QuantityId::DEVIATORIC_STRESS, QuantityId::DAMAGE }) {
            minimals.push_back(mv->minimal(id));
        }
    }
    w.u32("mat", mat);
    w.f64("mat_ranges", ranges);
    w.f64("mat_young", young);
    w.f64("mat_minimals", minimals);
}

void randomVelocities(Storage& s, uint64_t seed, double sigma) {
    SplitMix rng{ seed };
    ArrayView<Vector> v = s.getDt<Vector>(QuantityId::POSITION);
    for (Size i = 0; i < v.size(); ++i) {
        const double x = rng.normal(), y = rng.normal(), z = rng.normal();
        v[i] = Vector(sigma * x, sigma * y, sigma * z, 0._f);
    }
}

// Trajectory runs at the benchmark's sizes ("<kind>_traj" modes): every gDumpEvery steps (and after the first)
// the state of a seeded sample of gSample particles, the maximum magnitude, sum and sum of squares of every
// component over all particles, and the reference's integrals, so that a fixture stays small at 10^5 particles.
int gDumpEvery = 0;
int gSample = 0;
// frame frequency of the second set of integrals (TotalMomentum / TotalAngularMomentum / TotalEnergy(omega))
constexpr double TRAJ_FRAME_OMEGA = 1.e-4;

struct Sampler {
    std::vector<Size> idx;
    void f64(Writer& w, const std::string& name, const std::vector<double>& all, int comps) {
        const Size n = all.size() / comps;
        std::vector<double> pick, mx(comps, 0.), sum(comps, 0.), sum2(comps, 0.);
        for (Size i : idx) {
            for (int c = 0; c < comps; ++c) {
                pick.push_back(all[comps * i + c]);
            }
        }
        for (Size i = 0; i < n; ++i) {
            for (int c = 0; c < comps; ++c) {
                const double x = all[comps * i + c];
                mx[c] = std::max(mx[c], std::fabs(x));
                sum[c] += x;
                sum2[c] += x * x;
            }
        }
        w.f64(name, pick);
        w.f64(name + "@max", mx);
        w.f64(name + "@sum", sum);
        w.f64(name + "@sum2", sum2);
    }
    void u32(Writer& w, const std::string& name, const std::vector<uint32_t>& all) {
        std::vector<uint32_t> pick;
        double sum = 0.;
        for (Size i : idx) {
            pick.push_back(all[i]);
        }
        for (uint32_t x : all) {
            sum += x;
        }
        w.u32(name, pick);
        w.scalar(name + "@sum", sum);
    }
};

void dumpIntegrals(Writer& w, const std::string& pre, const Storage& s) {
    for (int k = 0; k < 2; ++k) {
        const double omega = k == 0 ? 0. : TRAJ_FRAME_OMEGA;
        const std::string suffix = k == 0 ? "" : "_frame";
        const Vector p = TotalMomentum(omega).evaluate(s);
        const Vector L = TotalAngularMomentum(omega).evaluate(s);
        w.f64(pre + "momentum" + suffix, { p[X], p[Y], p[Z] });
        w.f64(pre + "angular_momentum" + suffix, { L[X], L[Y], L[Z] });
        w.scalar(pre + "energy" + suffix, TotalEnergy(omega).evaluate(s));
    }
    w.scalar(pre + "kinetic_energy", TotalKineticEnergy().evaluate(s));
    w.scalar(pre + "internal_energy", TotalInternalEnergy().evaluate(s));
}

void dumpSampled(Writer& w, const std::string& pre, Storage& s, Sampler& smp) {
    ArrayView<const Vector> r, v, dv;
    tie(r, v, dv) = s.getAll<Vector>(QuantityId::POSITION);
    smp.f64(w, pre + "r", vec4(r), 4);
    smp.f64(w, pre + "v", vec4(v), 4);
    smp.f64(w, pre + "dv", vec4(dv), 4);
    {
        ArrayView<const Float> rho, drho;
        tie(rho, drho) = s.getAll<Float>(QuantityId::DENSITY);
        smp.f64(w, pre + "rho", flt(rho), 1);
        smp.f64(w, pre + "drho", flt(drho), 1);
    }
    {
        ArrayView<const Float> u, du;
        tie(u, du) = s.getAll<Float>(QuantityId::ENERGY);
        smp.f64(w, pre + "u", flt(u), 1);
        smp.f64(w, pre + "du", flt(du), 1);
    }
    smp.f64(w, pre + "p", flt(s.getValue<Float>(QuantityId::PRESSURE)), 1);
    smp.f64(w, pre + "cs", flt(s.getValue<Float>(QuantityId::SOUND_SPEED)), 1);
    if (s.has(QuantityId::NEIGHBOR_CNT)) {
        smp.u32(w, pre + "ncnt", sz(s.getValue<Size>(QuantityId::NEIGHBOR_CNT)));
    }
    if (s.has(QuantityId::DEVIATORIC_STRESS)) {
        ArrayView<const TracelessTensor> S, dS;
        tie(S, dS) = s.getAll<TracelessTensor>(QuantityId::DEVIATORIC_STRESS);
        smp.f64(w, pre + "S", traceless(S), 5);
        smp.f64(w, pre + "dS", traceless(dS), 5);
    }
    if (s.has(QuantityId::DAMAGE)) {
        ArrayView<const Float> D, dD;
        tie(D, dD) = s.getAll<Float>(QuantityId::DAMAGE);
        smp.f64(w, pre + "D", flt(D), 1);
        smp.f64(w, pre + "dD", flt(dD), 1);
    }
    dumpIntegrals(w, pre, s);
}

// Runs `steps` time steps, dumping the state after the first step and at the end, plus the dt sequence.
void runSteps(Writer& w, RunSettings& settings, SharedPtr<Storage> storage, int steps);

// Trajectory variant of runSteps: the full initial state, then sampled dumps (see Sampler) after step 1 and
// every gDumpEvery steps.
void runTrajectory(Writer& w, RunSettings& settings, SharedPtr<Storage> storage, int steps) {
    SharedPtr<IScheduler> scheduler = Factory::getScheduler(settings);
    AutoPtr<ISolver> solver = Factory::getSolver(*scheduler, settings);
    for (Size k = 0; k < storage->getMaterialCnt(); ++k) {
        solver->create(*storage, storage->getMaterial(k));
    }
    dumpMaterials(w, *storage);
    const Size n = storage->getParticleCnt();
    Sampler smp;
    {
        // gSample distinct indices, sorted; a seeded partial Fisher-Yates shuffle
        SplitMix rng{ 99 };
        std::vector<Size> perm(n);
        for (Size i = 0; i < n; ++i) {
            perm[i] = i;
        }
        const Size k = std::min<Size>(Size(gSample), n);
        for (Size i = 0; i < k; ++i) {
            const Size j = i + Size(rng.next() % uint64_t(n - i));
            std::swap(perm[i], perm[j]);
        }
        smp.idx.assign(perm.begin(), perm.begin() + k);
        std::sort(smp.idx.begin(), smp.idx.end());
        w.u32("sample_idx", std::vector<uint32_t>(smp.idx.begin(), smp.idx.end()));
    }
    {
        AutoPtr<ISolver> probeSolver = Factory::getSolver(*scheduler, settings);
        Storage probe = storage->clone(VisitorEnum::ALL_BUFFERS);
        probe.zeroHighestDerivatives(*scheduler);
        Statistics stats;
        stats.set(StatisticsId::RUN_TIME, 0._f);
        probeSolver->integrate(probe, stats);
        dumpSampled(w, "d0_", probe, smp);
    }
    AutoPtr<ITimeStepping> ts = Factory::getTimeStepping(settings, storage);
    dumpState(w, "s0_", *storage);
    dumpIntegrals(w, "s0_", *storage);
    std::vector<double> dts;
    std::vector<uint32_t> dumped;
    Statistics stats;
    double t = 0.;
    for (int step = 0; step < steps; ++step) {
        dts.push_back(ts->getTimeStep());
        stats.set(StatisticsId::RUN_TIME, t);
        t += ts->getTimeStep();
        ts->step(*scheduler, *solver, stats);
        const int done = step + 1;
        if (done == 1 || done % gDumpEvery == 0 || done == steps) {
            dumpSampled(w, "t" + std::to_string(done) + "_", *storage, smp);
            dumped.push_back(uint32_t(done));
        }
    }
    dts.push_back(ts->getTimeStep());
    w.f64("dts", dts);
    w.u32("dumped_steps", dumped);
}

void runSteps(Writer& w, RunSettings& settings, SharedPtr<Storage> storage, int steps) {
    if (gDumpEvery > 0) {
        runTrajectory(w, settings, storage, steps);
        return;
    }
    SharedPtr<IScheduler> scheduler = Factory::getScheduler(settings);
    AutoPtr<ISolver> solver = Factory::getSolver(*scheduler, settings);
    for (Size k = 0; k < storage->getMaterialCnt(); ++k) {
        solver->create(*storage, storage->getMaterial(k));
    }
    dumpMaterials(w, *storage);

    // one derivative evaluation on a copy of the initial state (ISolver::integrate alone), on a solver of its own
    // (a cached gravity would otherwise keep its accelerations)
    {
        AutoPtr<ISolver> probeSolver = Factory::getSolver(*scheduler, settings);
        Storage probe = storage->clone(VisitorEnum::ALL_BUFFERS);
        probe.zeroHighestDerivatives(*scheduler);
        Statistics stats;
        stats.set(StatisticsId::RUN_TIME, 0._f);
        probeSolver->integrate(probe, stats);
        dumpState(w, "d0_", probe);
    }

    AutoPtr<ITimeStepping> ts = Factory::getTimeStepping(settings, storage);
    dumpState(w, "s0_", *storage);
    std::vector<double> dts;
    Statistics stats;
    double t = 0.;
    for (int step = 0; step < steps; ++step) {
        dts.push_back(ts->getTimeStep());
        // the run time of the step, as the run loop sets it (core/run/IRun.cpp), read by CachedGravity
        stats.set(StatisticsId::RUN_TIME, t);
        t += ts->getTimeStep();
        ts->step(*scheduler, *solver, stats);
        if (step == 0) {
            dumpState(w, "s1_", *storage);
        }
    }
    dts.push_back(ts->getTimeStep());
    w.f64("dts", dts);
    dumpState(w, "sN_", *storage);
}

// the time-step criteria of the golden runs: COURANT, or every criterion (the reference's default ALL) when
// the mode name ends in "_all"
bool gAllCriteria = false;
// the AsymmetricSolver with the strain-rate correction tensor (mode name ending in "_asym")
bool gAsymmetric = false;
// CachedGravity with this recomputation period (mode name ending in "_cached"; the period is the last argument)
double gRecomputationPeriod = 0.;

RunSettings baseSettings() {
    RunSettings settings;
    settings.set(RunSettingsId::RUN_THREAD_CNT, 1);
    settings.set(RunSettingsId::SPH_AV_ALPHA, 1.5_f);
    settings.set(RunSettingsId::SPH_AV_BETA, 3._f);
    settings.set(RunSettingsId::SPH_FINDER, FinderEnum::KD_TREE);
    settings.set(RunSettingsId::GRAVITY_SOLVER, GravityEnum::BARNES_HUT);
    settings.set(RunSettingsId::GRAVITY_OPENING_ANGLE, 0.5_f);
    settings.set(RunSettingsId::GRAVITY_MULTIPOLE_ORDER, 3);
    settings.set(RunSettingsId::GRAVITY_KERNEL, GravityKernelEnum::SPH_KERNEL);
    settings.set(RunSettingsId::TIMESTEPPING_INTEGRATOR, TimesteppingEnum::PREDICTOR_CORRECTOR);
    if (gAllCriteria) {
        settings.set(RunSettingsId::TIMESTEPPING_CRITERION, TimeStepCriterionEnum::ALL);
    } else {
        settings.set(RunSettingsId::TIMESTEPPING_CRITERION, TimeStepCriterionEnum::COURANT);
    }
    if (gAsymmetric) {
        settings.set(RunSettingsId::SPH_SOLVER_TYPE, SolverEnum::ASYMMETRIC_SOLVER);
        settings.set(RunSettingsId::SPH_STRAIN_RATE_CORRECTION_TENSOR, true);
    }
    if (gRecomputationPeriod > 0.) {
        settings.set(RunSettingsId::GRAVITY_RECOMPUTATION_PERIOD, gRecomputationPeriod);
    }
    return settings;
}

// basalt sphere: Tillotson, Continuity + Pressure + StandardAV, BH gravity, constant h, PC, Courant
int modeSphere(Writer& w, int n, double radius, int steps, uint64_t seed) {
    RunSettings settings = baseSettings();
    settings.set(RunSettingsId::SPH_SOLVER_FORCES, ForceEnum::PRESSURE | ForceEnum::SELF_GRAVITY);
    settings.set(RunSettingsId::SPH_ADAPTIVE_SMOOTHING_LENGTH, EMPTY_FLAGS);
    BodySettings body;
    body.set(BodySettingsId::PARTICLE_COUNT, n);
    body.set(BodySettingsId::DENSITY, 2700._f);
    body.set(BodySettingsId::ENERGY, 1.e3_f);
    body.set(BodySettingsId::SMOOTHING_LENGTH_ETA, 1.43_f);
    body.set(BodySettingsId::EOS, EosEnum::TILLOTSON);
    body.set(BodySettingsId::RHEOLOGY_YIELDING, YieldingEnum::NONE);
    body.set(BodySettingsId::RHEOLOGY_DAMAGE, FractureEnum::NONE);
    SharedPtr<Storage> storage = makeShared<Storage>();
    InitialConditions ic(settings);
    ic.addMonolithicBody(*storage, SphericalDomain(Vector(0._f), radius), body);
    randomVelocities(*storage, seed, 1.0);
    w.scalar("G", settings.get<Float>(RunSettingsId::GRAVITY_CONSTANT));
    runSteps(w, settings, storage, steps);
    return 0;
}

// solid impact: target + impactor of basalt, Hooke + von Mises + Grady-Kipp, adaptive h, BH, PC, Courant
int modeImpact(Writer& w, int nt, double rt, int ni, double ri, int steps, double speed, double angleDeg) {
    RunSettings settings = baseSettings();
    settings.set(RunSettingsId::SPH_SOLVER_FORCES,
        ForceEnum::PRESSURE | ForceEnum::SOLID_STRESS | ForceEnum::SELF_GRAVITY);
    settings.set(RunSettingsId::SPH_ADAPTIVE_SMOOTHING_LENGTH, SmoothingLengthEnum::CONTINUITY_EQUATION);
    BodySettings body;
    body.set(BodySettingsId::DENSITY, 2700._f);
    body.set(BodySettingsId::EOS, EosEnum::TILLOTSON);
    body.set(BodySettingsId::RHEOLOGY_YIELDING, YieldingEnum::VON_MISES);
    body.set(BodySettingsId::RHEOLOGY_DAMAGE, FractureEnum::SCALAR_GRADY_KIPP);
    SharedPtr<Storage> storage = makeShared<Storage>();
    InitialConditions ic(settings);
    body.set(BodySettingsId::PARTICLE_COUNT, nt);
    ic.addMonolithicBody(*storage, SphericalDomain(Vector(0._f), rt), body);
    const Float h = storage->getValue<Vector>(QuantityId::POSITION)[0][H];
    const Float phi = angleDeg * DEG_TO_RAD;
    const Float dist = rt + ri;
    const Vector center(dist * std::cos(phi) + 4._f * h, dist * std::sin(phi), 0._f);
    body.set(BodySettingsId::PARTICLE_COUNT, ni);
    ic.addMonolithicBody(*storage, SphericalDomain(center, ri), body).addVelocity(Vector(-speed, 0._f, 0._f));
    w.scalar("G", settings.get<Float>(RunSettingsId::GRAVITY_CONSTANT));
    runSteps(w, settings, storage, steps);
    return 0;
}

// ideal gas sphere + Mach-3 impactor: Continuity + Pressure + StandardAV, leap-frog, no gravity
int modeGas(Writer& w, int nt, int ni, int steps) {
    RunSettings settings = baseSettings();
    settings.set(RunSettingsId::SPH_SOLVER_FORCES, ForceEnum::PRESSURE);
    settings.set(RunSettingsId::SPH_ADAPTIVE_SMOOTHING_LENGTH, EMPTY_FLAGS);
    settings.set(RunSettingsId::TIMESTEPPING_INTEGRATOR, TimesteppingEnum::LEAP_FROG);
    settings.set(RunSettingsId::TIMESTEPPING_INITIAL_TIMESTEP, 1.e-3_f);
    BodySettings body;
    body.set(BodySettingsId::EOS, EosEnum::IDEAL_GAS);
    body.set(BodySettingsId::ADIABATIC_INDEX, 5._f / 3._f);
    body.set(BodySettingsId::DENSITY, 1._f);
    body.set(BodySettingsId::DENSITY_RANGE, Interval(1.e-3_f, INFTY));
    body.set(BodySettingsId::ENERGY, 1.5_f);
    body.set(BodySettingsId::RHEOLOGY_YIELDING, YieldingEnum::NONE);
    body.set(BodySettingsId::RHEOLOGY_DAMAGE, FractureEnum::NONE);
    SharedPtr<Storage> storage = makeShared<Storage>();
    InitialConditions ic(settings);
    body.set(BodySettingsId::PARTICLE_COUNT, nt);
    ic.addMonolithicBody(*storage, SphericalDomain(Vector(0._f), 1._f), body);
    body.set(BodySettingsId::PARTICLE_COUNT, ni);
    const Float cs = std::sqrt(5._f / 3._f);
    ic.addMonolithicBody(*storage, SphericalDomain(Vector(1.35_f, 0.3_f, 0._f), 0.25_f), body)
        .addVelocity(Vector(-3._f * cs, 0._f, 0._f));
    runSteps(w, settings, storage, steps);
    return 0;
}

// gravity only: Barnes-Hut (octupole, SPH gravity kernel, leaf 25) and brute force on seeded points
int modeGravity(Writer& w, int n, double theta, uint64_t seed, double soft) {
    SplitMix rng{ seed };
    Array<Vector> r(n);
    Array<Float> m(n);
    for (int i = 0; i < n; ++i) {
        // Plummer sphere, scale radius 1, radius capped at 10
        double rad;
        do {
            const double x = rng.uniform();
            rad = 1.0 / std::sqrt(std::pow(x, -2.0 / 3.0) - 1.0);
        } while (rad > 10.0);
        const double ct = 2.0 * rng.uniform() - 1.0;
        const double ph = 2.0 * 3.14159265358979323846 * rng.uniform();
        const double st = std::sqrt(1.0 - ct * ct);
        r[i] = Vector(rad * st * std::cos(ph), rad * st * std::sin(ph), rad * ct, soft);
        m[i] = 1.0 / n;
    }
    Storage storage;
    storage.insert<Vector>(QuantityId::POSITION, OrderEnum::SECOND, r.clone());
    storage.insert<Float>(QuantityId::MASS, OrderEnum::ZERO, m.clone());
    w.f64("r", vec4(r));
    w.f64("m", flt(m));
    BarnesHut bh(theta, MultipoleOrder::OCTUPOLE, GravityKernel<CubicSpline<3>>{}, 25, 50, 1._f);
    bh.build(SEQUENTIAL, storage);
    Array<Vector> dv(n);
    dv.fill(Vector(0._f));
    Statistics stats;
    bh.evalSelfGravity(SEQUENTIAL, dv, stats);
    w.f64("a_bh", vec4(dv));
    w.scalar("nodes_approx", stats.get<int>(StatisticsId::GRAVITY_NODES_APPROX));
    w.scalar("nodes_exact", stats.get<int>(StatisticsId::GRAVITY_NODES_EXACT));
    w.scalar("node_count", stats.get<int>(StatisticsId::GRAVITY_NODE_COUNT));
    BruteForceGravity bf(GravityKernel<CubicSpline<3>>{}, 1._f);
    bf.build(SEQUENTIAL, storage);
    Array<Vector> dvb(n);
    dvb.fill(Vector(0._f));
    bf.evalSelfGravity(SEQUENTIAL, dvb, stats);
    w.f64("a_direct", vec4(dvb));
    const MultipoleExpansion<3> root = bh.getMoments();
    std::vector<double> mom;
    mom.push_back(root.order<0>().value());
    w.f64("root_m0", mom);
    return 0;
}

// BarnesHut::evalAttractors (core/gravity/BarnesHut.cpp:100-125) on a Plummer sphere with two attractors (one
// inside the particle cloud, one outside): the particles' accelerations (self-gravity, then the attractor terms
// added) and the attractors' accelerations
int modeAttractors(Writer& w, int n, uint64_t seed, double soft) {
    SplitMix rng{ seed };
    Array<Vector> r(n);
    Array<Float> m(n);
    for (int i = 0; i < n; ++i) {
        double rad;
        do {
            const double x = rng.uniform();
            rad = 1.0 / std::sqrt(std::pow(x, -2.0 / 3.0) - 1.0);
        } while (rad > 10.0);
        const double ct = 2.0 * rng.uniform() - 1.0;
        const double ph = 2.0 * 3.14159265358979323846 * rng.uniform();
        const double st = std::sqrt(1.0 - ct * ct);
        r[i] = Vector(rad * st * std::cos(ph), rad * st * std::sin(ph), rad * ct, soft);
        m[i] = 1.0 / n;
    }
    Storage storage;
    storage.insert<Vector>(QuantityId::POSITION, OrderEnum::SECOND, r.clone());
    storage.insert<Float>(QuantityId::MASS, OrderEnum::ZERO, m.clone());
    w.f64("r", vec4(r));
    w.f64("m", flt(m));
    const double G = 0.7;
    BarnesHut bh(0.5, MultipoleOrder::OCTUPOLE, GravityKernel<CubicSpline<3>>{}, 25, 50, G);
    bh.build(SEQUENTIAL, storage);
    Array<Vector> dv(n);
    dv.fill(Vector(0._f));
    Statistics stats;
    bh.evalSelfGravity(SEQUENTIAL, dv, stats);
    w.f64("a_self", vec4(dv));
    Array<Attractor> attractors;
    attractors.push(Attractor(Vector(0.1, -0.2, 0.05), Vector(0._f), 0.3, 0.25));
    attractors.push(Attractor(Vector(4.0, 3.0, -2.0), Vector(0._f), 0.5, 2.0));
    std::vector<double> att;
    for (const Attractor& a : attractors) {
        att.insert(att.end(), { a.position[X], a.position[Y], a.position[Z], a.radius, a.mass });
    }
    bh.evalAttractors(SEQUENTIAL, attractors, dv);
    std::vector<double> aacc;
    for (const Attractor& a : attractors) {
        aacc.insert(aacc.end(), { a.acceleration[X], a.acceleration[Y], a.acceleration[Z] });
    }
    w.scalar("G", G);
    w.f64("attractors", att);
    w.f64("a_total", vec4(dv));
    w.f64("attractor_acc", aacc);
    return 0;
}

// BruteForceGravity (core/gravity/BruteForceGravity.h:38-58, 110-129) on n seeded points whose coordinates use only
// exactly rounded arithmetic, so that any machine regenerates them bit for bit: per coordinate x = s (2u - 1) with
// s = u'^2 (u, u' uniform from the splitmix64 sequence, one u' per point), h = soft, m = 1 / n, G = 1; writes the
// accelerations of nSample seeded particles and checksums of the points.
int modeDirect(Writer& w, int n, uint64_t seed, double soft, int nSample) {
    SplitMix rng{ seed };
    Array<Vector> r(n);
    Array<Float> m(n);
    double sx = 0., sy = 0., sz = 0.;
    for (int i = 0; i < n; ++i) {
        const double u = rng.uniform();
        const double s = u * u;
        const double x = s * (2. * rng.uniform() - 1.);
        const double y = s * (2. * rng.uniform() - 1.);
        const double z = s * (2. * rng.uniform() - 1.);
        r[i] = Vector(x, y, z, soft);
        m[i] = 1. / n;
        sx += x;
        sy += y;
        sz += z;
    }
    Storage storage;
    storage.insert<Vector>(QuantityId::POSITION, OrderEnum::SECOND, r.clone());
    storage.insert<Float>(QuantityId::MASS, OrderEnum::ZERO, m.clone());
    BruteForceGravity bf(GravityKernel<CubicSpline<3>>{}, 1._f);
    bf.build(SEQUENTIAL, storage);
    Array<Vector> dv(n);
    dv.fill(Vector(0._f));
    Statistics stats;
    bf.evalSelfGravity(SEQUENTIAL, dv, stats);
    SplitMix pick{ seed + 1 };
    std::vector<uint32_t> idx;
    std::vector<double> acc;
    for (int k = 0; k < nSample; ++k) {
        const uint32_t i = uint32_t(pick.next() % uint64_t(n));
        idx.push_back(i);
        for (int c = 0; c < 4; ++c) {
            acc.push_back(dv[i][c]);
        }
    }
    w.f64("params", { double(n), double(seed), soft });
    w.f64("checksum", { sx, sy, sz });
    w.u32("sample_idx", idx);
    w.f64("a_direct", acc);
    return 0;
}

// symmetric-finder pair set (KdTree.findLowerRank + the SymmetricSolver radius filter) on a solver state
int modePairs(Writer& w, int n, uint64_t seed) {
    SplitMix rng{ seed };
    Array<Vector> r(n);
    for (int i = 0; i < n; ++i) {
        const double x = rng.uniform(), y = rng.uniform(), z = rng.uniform();
        const double h = 0.05 + 0.05 * rng.uniform();
        r[i] = Vector(x, y, z, h);
    }
    w.f64("r", vec4(r));
    KdTree<KdNode> tree;
    tree.build(SEQUENTIAL, r, FinderFlag::MAKE_RANK);
    Array<NeighborRecord> neighs;
    std::vector<uint32_t> pi, pj;
    for (int i = 0; i < n; ++i) {
        tree.findLowerRank(i, 2._f * r[i][H], neighs);
        for (const NeighborRecord& nr : neighs) {
            const Size j = nr.index;
            const Float hbar = 0.5_f * (r[i][H] + r[j][H]);
            if (getSqrLength(r[i] - r[j]) >= sqr(2._f * hbar)) {
                continue;
            }
            pi.push_back(i);
            pj.push_back(j);
        }
    }
    w.u32("pair_i", pi);
    w.u32("pair_j", pj);
    return 0;
}

// known-answer values of the EOS
int modeEos(Writer& w) {
    BodySettings settings;
    settings.set(BodySettingsId::DENSITY, 2.7_f);
    settings.set(BodySettingsId::TILLOTSON_SUBLIMATION, 1.e5_f);
    TillotsonEos eos(settings);
    std::vector<double> rho, u, p, cs;
    for (double rr : { 1.0, 2.0, 2.6, 2.7, 2.8, 3.5 }) {
        for (double uu : { 1.e3, 1.e5, 1.e7, 1.e10 }) {
            Float pp, cc;
            tie(pp, cc) = eos.evaluate(rr, uu);
            rho.push_back(rr);
            u.push_back(uu);
            p.push_back(pp);
            cs.push_back(cc);
        }
    }
    w.f64("rho", rho);
    w.f64("u", u);
    w.f64("p", p);
    w.f64("cs", cs);
    return 0;
}

} // namespace

// HardSphereSolver wrapper that sums the collision statistics of every collide() call (the reference sets
// them per call, core/gravity/NBodySolver.cpp:119-163)
void dumpNbody(Writer& w, const std::string& pre, Storage& s);

class CountingSolver : public ISolver {
public:
    HardSphereSolver inner;
    std::vector<double> totals = std::vector<double>(4, 0.);
    // the states before and after the collide calls from call number traceFrom on are written to trace
    Writer* trace = nullptr;
    int traceFrom = 1 << 30;
    int calls = 0;

    CountingSolver(IScheduler& scheduler, const RunSettings& settings)
        : inner(scheduler, settings) {}

    virtual void integrate(Storage& storage, Statistics& stats) override {
        inner.integrate(storage, stats);
    }
    virtual void collide(Storage& storage, Statistics& stats, const Float dt) override {
        const StatisticsId ids[4] = { StatisticsId::TOTAL_COLLISION_COUNT, StatisticsId::MERGER_COUNT,
            StatisticsId::BOUNCE_COUNT, StatisticsId::OVERLAP_COUNT };
        for (StatisticsId id : ids) {
            stats.set(id, 0);
        }
        const bool traced = trace && calls >= traceFrom;
        if (traced) {
            dumpNbody(*trace, "pre" + std::to_string(calls) + "_", storage);
            trace->scalar("dt" + std::to_string(calls), dt);
        }
        inner.collide(storage, stats, dt);
        if (traced) {
            dumpNbody(*trace, "post" + std::to_string(calls) + "_", storage);
        }
        ++calls;
        for (int k = 0; k < 4; ++k) {
            totals[k] += stats.get<int>(ids[k]);
        }
    }
    virtual void create(Storage& storage, IMaterial& material) const override {
        inner.create(storage, material);
    }
};

void dumpNbody(Writer& w, const std::string& pre, Storage& s) {
    ArrayView<const Vector> r, v, dv;
    tie(r, v, dv) = s.getAll<Vector>(QuantityId::POSITION);
    w.f64(pre + "r", vec4(r));
    w.f64(pre + "v", vec4(v));
    w.f64(pre + "dv", vec4(dv));
    w.f64(pre + "m", flt(s.getValue<Float>(QuantityId::MASS)));
    w.f64(pre + "w", vec4(s.getValue<Vector>(QuantityId::ANGULAR_FREQUENCY)));
}

// N-body cloud: n hard spheres of radius h (times 1 + 0.5 u, u uniform in [0, 1)) and density 2500, placed
// uniformly in a sphere of radius R without overlaps, moving inward with velocity -k r plus a normal
// velocity dispersion sigma; HardSphereSolver with BH self-gravity (solid spheres, theta 0.8, leaf 20),
// leap-frog with the acceleration criterion (factor 0.2), the N-body run's settings otherwise
// (core/run/jobs/SimulationJobs.cpp:462-494) except the handlers given here.
int modeNbody(Writer& w, int n, int steps, int handler, int overlap, double R, double h, double k, double sigma,
    uint64_t seed, double G, double maxDt) {
    RunSettings settings;
    settings.set(RunSettingsId::RUN_THREAD_CNT, 1);
    settings.set(RunSettingsId::SPH_FINDER, FinderEnum::KD_TREE);
    settings.set(RunSettingsId::FINDER_LEAF_SIZE, 20);
    settings.set(RunSettingsId::GRAVITY_SOLVER, GravityEnum::BARNES_HUT);
    settings.set(RunSettingsId::GRAVITY_KERNEL, GravityKernelEnum::SOLID_SPHERES);
    settings.set(RunSettingsId::GRAVITY_OPENING_ANGLE, 0.8_f);
    settings.set(RunSettingsId::GRAVITY_MULTIPOLE_ORDER, 3);
    settings.set(RunSettingsId::GRAVITY_CONSTANT, G);
    settings.set(RunSettingsId::COLLISION_HANDLER, CollisionHandlerEnum(handler));
    settings.set(RunSettingsId::COLLISION_OVERLAP, OverlapEnum(overlap));
    settings.set(RunSettingsId::COLLISION_RESTITUTION_NORMAL, 0.5_f);
    settings.set(RunSettingsId::COLLISION_RESTITUTION_TANGENT, 1._f);
    settings.set(RunSettingsId::COLLISION_ALLOWED_OVERLAP, 0.01_f);
    settings.set(RunSettingsId::COLLISION_BOUNCE_MERGE_LIMIT, 4._f);
    settings.set(RunSettingsId::COLLISION_ROTATION_MERGE_LIMIT, 1._f);
    settings.set(RunSettingsId::NBODY_INERTIA_TENSOR, false);
    settings.set(RunSettingsId::TIMESTEPPING_INITIAL_TIMESTEP, maxDt);
    settings.set(RunSettingsId::TIMESTEPPING_MAX_TIMESTEP, maxDt);
    settings.set(RunSettingsId::TIMESTEPPING_CRITERION, TimeStepCriterionEnum::ACCELERATION);
    settings.set(RunSettingsId::TIMESTEPPING_DERIVATIVE_FACTOR, 0.2_f);

    SplitMix rng{ seed };
    Array<Vector> r;
    Array<Float> m;
    while (r.size() < Size(n)) {
        const double x = (2. * rng.uniform() - 1.) * R, y = (2. * rng.uniform() - 1.) * R,
                     z = (2. * rng.uniform() - 1.) * R;
        if (x * x + y * y + z * z > R * R) {
            continue;
        }
        const double hi = h * (1. + 0.5 * rng.uniform());
        bool free = true;
        for (Size j = 0; j < r.size() && free; ++j) {
            const double dx = r[j][X] - x, dy = r[j][Y] - y, dz = r[j][Z] - z;
            free = dx * dx + dy * dy + dz * dz > (hi + r[j][H]) * (hi + r[j][H]);
        }
        if (free) {
            r.push(Vector(x, y, z, hi));
            m.push(2500. * 4. / 3. * 3.14159265358979323846 * hi * hi * hi);
        }
    }
    Array<Vector> v(r.size());
    for (Size i = 0; i < r.size(); ++i) {
        v[i] = Vector(-k * r[i][X] + sigma * rng.normal(), -k * r[i][Y] + sigma * rng.normal(),
            -k * r[i][Z] + sigma * rng.normal(), 0._f);
    }
    SharedPtr<Storage> storage = makeShared<Storage>(makeAuto<NullMaterial>(BodySettings::getDefaults()));
    storage->insert<Vector>(QuantityId::POSITION, OrderEnum::SECOND, std::move(r));
    storage->getDt<Vector>(QuantityId::POSITION).fill(Vector(0._f));
    {
        ArrayView<Vector> vv = storage->getDt<Vector>(QuantityId::POSITION);
        for (Size i = 0; i < vv.size(); ++i) {
            vv[i] = v[i];
        }
    }
    storage->insert<Float>(QuantityId::MASS, OrderEnum::ZERO, std::move(m));
    SharedPtr<IScheduler> scheduler = Factory::getScheduler(settings);
    CountingSolver solver(*scheduler, settings);
    solver.create(*storage, storage->getMaterial(0));
    if (std::getenv("NBODY_TRACE_LAST_STEP")) {
        solver.trace = &w;
        solver.traceFrom = 2 * (steps - 1);
    }
    w.scalar("G", G);
    w.f64("settings", { double(handler), double(overlap), 0.5, 1., 0.01, 4., 1., 0.8, 20., maxDt, 0.2 });
    dumpNbody(w, "s0_", *storage);
    LeapFrog ts(storage, settings);
    Statistics stats;
    std::vector<double> dts, counts;
    for (int step = 0; step < steps; ++step) {
        dts.push_back(ts.getTimeStep());
        ts.step(*scheduler, solver, stats);
        counts.push_back(double(storage->getParticleCnt()));
        if (step == 0) {
            dumpNbody(w, "s1_", *storage);
        }
    }
    dts.push_back(ts.getTimeStep());
    w.f64("dts", dts);
    w.f64("counts", counts);
    w.f64("collision_stats", solver.totals);
    dumpNbody(w, "sN_", *storage);
    return 0;
}

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: refdriver <out> <mode> [args]\n");
        return 2;
    }
    Writer w(argv[1]);
    std::string mode = argv[2];
    if (mode.size() > 4 && mode.compare(mode.size() - 4, 4, "_all") == 0) {
        gAllCriteria = true;
        mode = mode.substr(0, mode.size() - 4);
    }
    if (mode.size() > 7 && mode.compare(mode.size() - 7, 7, "_cached") == 0) {
        gRecomputationPeriod = std::atof(argv[argc - 1]);
        --argc;
        mode = mode.substr(0, mode.size() - 7);
    }
    if (mode.size() > 5 && mode.compare(mode.size() - 5, 5, "_asym") == 0) {
        gAsymmetric = true;
        mode = mode.substr(0, mode.size() - 5);
    }
    if (mode.size() > 5 && mode.compare(mode.size() - 5, 5, "_traj") == 0) {
        // the last two arguments: dump interval and sample size
        gSample = std::atoi(argv[argc - 1]);
        gDumpEvery = std::atoi(argv[argc - 2]);
        argc -= 2;
        mode = mode.substr(0, mode.size() - 5);
        if (gDumpEvery <= 0 || gSample <= 0) {
            std::fprintf(stderr, "trajectory mode needs a positive dump interval and sample size\n");
            return 2;
        }
    }
    auto arg = [&](int k, double dflt) { return argc > k ? std::atof(argv[k]) : dflt; };
    try {
        if (mode == "sphere") {
            return modeSphere(w, int(arg(3, 1000)), arg(4, 1.e4), int(arg(5, 5)), uint64_t(arg(6, 1)));
        } else if (mode == "impact") {
            return modeImpact(w,
                int(arg(3, 2000)),
                arg(4, 5.e4),
                int(arg(5, 100)),
                arg(6, 5.e3),
                int(arg(7, 5)),
                arg(8, 5.e3),
                arg(9, 45.));
        } else if (mode == "gas") {
            return modeGas(w, int(arg(3, 2000)), int(arg(4, 100)), int(arg(5, 5)));
        } else if (mode == "gravity") {
            return modeGravity(w, int(arg(3, 2000)), arg(4, 0.5), uint64_t(arg(5, 7)), arg(6, 1.e-3));
        } else if (mode == "attractors") {
            return modeAttractors(w, int(arg(3, 2000)), uint64_t(arg(4, 7)), arg(5, 1.e-2));
        } else if (mode == "direct") {
            return modeDirect(w, int(arg(3, 65536)), uint64_t(arg(4, 17)), arg(5, 1.e-3), int(arg(6, 1024)));
        } else if (mode == "pairs") {
            return modePairs(w, int(arg(3, 1000)), uint64_t(arg(4, 3)));
        } else if (mode == "eos") {
            return modeEos(w);
        } else if (mode == "nbody") {
            return modeNbody(w, int(arg(3, 1000)), int(arg(4, 20)), int(arg(5, 3)), int(arg(6, 5)), arg(7, 2000.),
                arg(8, 40.), arg(9, 1.e-3), arg(10, 0.05), uint64_t(arg(11, 5)), arg(12, 6.67408e-11),
                arg(13, 10.));
        }
    } catch (const std::exception& e) {
        std::fprintf(stderr, "reference threw: %s\n", e.what());
        return 1;
    }
    std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
    return 2;
}
