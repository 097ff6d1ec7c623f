/// \file adaptor_check.cpp
/// \brief Builds the reference-side adaptors into a small OpenSPH program: the initial conditions of the
/// reference, GpuSolver::create, then one step through GpuTimeStepping. Without a CUDA device the step
/// must end in the reference's Exception type carrying the library's message (no crash, no fallback).
/// Exit code: 0 = completed a step on a GPU, 3 = clean "no device" exception, 1 = anything else.

#include "GpuSph.h"
#include "Sph.h"

#include <cstdio>

using namespace Sph;

int main() {
    RunSettings settings;
    settings.set(RunSettingsId::RUN_THREAD_CNT, 1);
    settings.set(RunSettingsId::SPH_SOLVER_FORCES, ForceEnum::PRESSURE | ForceEnum::SELF_GRAVITY);
    settings.set(RunSettingsId::SPH_ADAPTIVE_SMOOTHING_LENGTH, EMPTY_FLAGS);
    settings.set(RunSettingsId::TIMESTEPPING_CRITERION, TimeStepCriterionEnum::COURANT);
    BodySettings body;
    body.set(BodySettingsId::PARTICLE_COUNT, 2000);
    body.set(BodySettingsId::ENERGY, 1.e3_f);
    body.set(BodySettingsId::RHEOLOGY_YIELDING, YieldingEnum::NONE);
    body.set(BodySettingsId::RHEOLOGY_DAMAGE, FractureEnum::NONE);
    SharedPtr<Storage> storage = makeShared<Storage>();
    InitialConditions ic(settings);
    ic.addMonolithicBody(*storage, SphericalDomain(Vector(0._f), 1.e4_f), body);
    SharedPtr<IScheduler> scheduler = Factory::getScheduler(settings);
    Gpu::GpuSolver solver(*scheduler, settings);
    for (Size k = 0; k < storage->getMaterialCnt(); ++k) {
        solver.create(*storage, storage->getMaterial(k));
    }
    Gpu::GpuTimeStepping stepping(storage, settings);
    Statistics stats;
    try {
        stepping.step(*scheduler, solver, stats);
    } catch (const Exception& e) {
        std::printf("exception: %s\n", e.what());
        return std::string(e.what()).find("no CUDA device") != std::string::npos ? 3 : 1;
    }
    std::printf("step done: dt = %g\n", stepping.getTimeStep());
    return 0;
}
