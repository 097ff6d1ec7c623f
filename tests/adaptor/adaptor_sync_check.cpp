/// \file adaptor_sync_check.cpp
/// \brief The adaptor's host/device synchronisation, against the reference's own BinaryOutput / BinaryInput.
///
/// Linked with tests/adaptor/fake_sphgpu.cpp (host-memory stand-in for libsphgpu that drifts r += v dt per
/// step and counts position uploads and downloads). Checks, for GpuTimeStepping in ON_DEMAND mode: one upload
/// before the first step and no download between steps; GpuOutput downloads once before writing the .ssf;
/// the file read back by BinaryInput holds the device state; invalidate() (a resumed run) uploads again; and
/// EVERY_STEP mode downloads after every step. It also checks that GpuHardSphereSolver::collide removes the
/// particles merged on the device from the host Storage, in the numbering of each call. Prints "ok" and exits 0
/// on success.

#include "GpuSph.h"
#include "Sph.h"

#include <cmath>
#include <cstdio>

using namespace Sph;

extern "C" void fake_sphgpu_counts(int* uploads, int* downloads, int* steps);

namespace {

int fails = 0;

void expect(const bool cond, const char* what) {
    if (!cond) {
        std::printf("FAILED: %s\n", what);
        fails++;
    }
}

void counts(int& up, int& down, int& steps) {
    fake_sphgpu_counts(&up, &down, &steps);
}

} // namespace

int main(int argc, char** argv) {
    if (argc < 2) {
        std::printf("usage: adaptor_sync_check <output directory>\n");
        return 2;
    }
    const std::string dir = argv[1];
    RunSettings settings;
    settings.set(RunSettingsId::RUN_THREAD_CNT, 1);
    settings.set(RunSettingsId::SPH_SOLVER_FORCES, ForceEnum::PRESSURE);
    settings.set(RunSettingsId::SPH_ADAPTIVE_SMOOTHING_LENGTH, EMPTY_FLAGS);
    settings.set(RunSettingsId::TIMESTEPPING_CRITERION, TimeStepCriterionEnum::COURANT);
    settings.set(RunSettingsId::TIMESTEPPING_INITIAL_TIMESTEP, 0.01_f);
    BodySettings body;
    body.set(BodySettingsId::PARTICLE_COUNT, 500);
    body.set(BodySettingsId::EOS, EosEnum::IDEAL_GAS);
    body.set(BodySettingsId::DENSITY, 1._f);
    body.set(BodySettingsId::ENERGY, 1._f);
    body.set(BodySettingsId::RHEOLOGY_YIELDING, YieldingEnum::NONE);
    body.set(BodySettingsId::RHEOLOGY_DAMAGE, FractureEnum::NONE);
    SharedPtr<Storage> storage = makeShared<Storage>();
    InitialConditions ic(settings);
    ic.addMonolithicBody(*storage, SphericalDomain(Vector(0._f), 1._f), body).addVelocity(Vector(1._f, 2._f, 3._f));
    SharedPtr<IScheduler> scheduler = Factory::getScheduler(settings);
    Gpu::GpuSolver solver(*scheduler, settings);
    for (Size k = 0; k < storage->getMaterialCnt(); ++k) {
        solver.create(*storage, storage->getMaterial(k));
    }
    const Vector r0 = storage->getValue<Vector>(QuantityId::POSITION)[7];

    Gpu::GpuTimeStepping stepping(storage, settings, Gpu::SyncMode::ON_DEMAND);
    Gpu::GpuOutput output(makeAuto<BinaryOutput>(OutputFile(Path(String::fromAscii((dir + "/dump_%d.ssf").c_str())))), stepping);
    Statistics stats;
    stats.set(StatisticsId::RUN_TIME, 0._f);
    int up = 0, down = 0, steps = 0;
    for (int k = 0; k < 3; ++k) {
        stepping.step(*scheduler, solver, stats);
    }
    counts(up, down, steps);
    expect(up == 1 && down == 0 && steps == 3, "ON_DEMAND: one upload, no download in three steps");
    expect(storage->getValue<Vector>(QuantityId::POSITION)[7] == r0, "host storage untouched between outputs");

    const Expected<Path> path = output.dump(*storage, stats);
    expect(bool(path), "GpuOutput wrote the file");
    counts(up, down, steps);
    expect(down == 1, "GpuOutput synchronised once before the dump");
    const Vector r3 = storage->getValue<Vector>(QuantityId::POSITION)[7];
    expect(std::abs(r3[X] - (r0[X] + 3 * 0.01 * 1.)) < 1e-12 && std::abs(r3[Z] - (r0[Z] + 3 * 0.01 * 3.)) < 1e-12,
        "the synchronised storage holds the device state after three steps");
    output.dump(*storage, stats);
    counts(up, down, steps);
    expect(down == 1, "a second dump without a step does not synchronise again");

    // resume: the reference's BinaryInput reads the dump into a new storage, the run continues from it
    if (path) {
        Storage loaded;
        Statistics loadedStats;
        BinaryInput input;
        const Outcome result = input.load(path.value(), loaded, loadedStats);
        expect(bool(result), "BinaryInput loaded the dump");
        if (result) {
            expect(loaded.getParticleCnt() == storage->getParticleCnt(), "same particle count");
            expect(loaded.getValue<Vector>(QuantityId::POSITION)[7] == r3, "the file holds the device state");
        }
    }
    stepping.invalidate();
    stepping.step(*scheduler, solver, stats);
    counts(up, down, steps);
    expect(up == 2 && down == 1, "invalidate() uploads the host storage before the next step");

    // EVERY_STEP: the host storage follows the device after each step
    Gpu::GpuTimeStepping every(storage, settings, Gpu::SyncMode::EVERY_STEP);
    for (int k = 0; k < 2; ++k) {
        every.step(*scheduler, solver, stats);
    }
    int up2 = 0, down2 = 0, steps2 = 0;
    counts(up2, down2, steps2);
    expect(down2 - down == 2 && up2 - up == 2, "EVERY_STEP uploads and downloads once per step");
    expect(every.syncCount() == 2, "EVERY_STEP sync count");

    // N-body: GpuHardSphereSolver removes the particles merged on the device from the host Storage (the
    // stand-in merges every odd particle into its even neighbour)
    {
        RunSettings nb;
        nb.set(RunSettingsId::RUN_THREAD_CNT, 1);
        nb.set(RunSettingsId::COLLISION_HANDLER, CollisionHandlerEnum::PERFECT_MERGING);
        SharedPtr<Storage> s = makeShared<Storage>(makeAuto<NullMaterial>(BodySettings::getDefaults()));
        Array<Vector> r;
        Array<Float> m;
        for (Size i = 0; i < 7; ++i) {
            r.push(Vector(Float(i), 0._f, 0._f, 0.1_f));
            m.push(1._f + Float(i));
        }
        s->insert<Vector>(QuantityId::POSITION, OrderEnum::SECOND, std::move(r));
        s->insert<Float>(QuantityId::MASS, OrderEnum::ZERO, std::move(m));
        Gpu::GpuHardSphereSolver hs(*scheduler, nb);
        hs.create(*s, s->getMaterial(0));
        Statistics nstats;
        hs.collide(*s, nstats, 1._f);
        expect(s->getParticleCnt() == 4, "N-body: three merged particles removed from the Storage");
        ArrayView<const Vector> rr = s->getValue<Vector>(QuantityId::POSITION);
        ArrayView<const Float> mm = s->getValue<Float>(QuantityId::MASS);
        expect(rr[1][X] == 2._f && rr[3][X] == 6._f, "N-body: the order of the kept particles is unchanged");
        expect(mm[0] == 3._f && mm[3] == 7._f, "N-body: the merged masses are read back");
        expect(nstats.get<int>(StatisticsId::MERGER_COUNT) == 3, "N-body: merger count of the call");
        hs.collide(*s, nstats, 1._f);
        expect(s->getParticleCnt() == 2, "N-body: the second call removes relative to the new numbering");
    }

    if (fails == 0) {
        std::printf("ok\n");
        return 0;
    }
    return 1;
}
