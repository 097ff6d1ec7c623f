#pragma once
/// \file GpuSph.h
/// \brief Reference-side adaptors: OpenSPH interfaces implemented over the libsphgpu C ABI.
///
/// These classes are compiled inside an OpenSPH build (they include the reference's headers) and forward
/// the per-step hot path to the GB300 library through include/sphgpu.h:
///   - GpuSolver        : ISolver       (replaces GravitySolver<SymmetricSolver<3>>, Factory::getSolver)
///   - GpuTimeStepping  : ITimeStepping (PredictorCorrector / LeapFrog with the step on the device)
///   - GpuBarnesHut     : IGravity      (replaces BarnesHut, Factory::getGravity)
///   - GpuFinder        : ISymmetricFinder (replaces KdTree, Factory::getFinder)
///   - GpuOutput        : IOutput decorator bringing the host Storage up to date before each dump, so that
///                        the reference's BinaryOutput (.ssf) writes the device state without per-step syncs
///   - GpuHardSphereSolver : ISolver   (replaces HardSphereSolver, the N-body solver with collisions)
/// Errors reported by the library are rethrown as the reference's InvalidSetup (configuration) or
/// Exception (runtime) types.

#include "gravity/IGravity.h"
#include "io/Output.h"
#include "objects/finders/NeighborFinder.h"
#include "quantities/Storage.h"
#include "system/Settings.h"
#include "timestepping/ISolver.h"
#include "timestepping/TimeStepping.h"

#include "sphgpu.h"

#include <memory>
#include <vector>

NAMESPACE_SPH_BEGIN

namespace Gpu {

/// Owns one sphgpu handle (particle state in HBM) and moves Storage quantities across the C ABI.
class DeviceState {
    sphgpu_handle* handle = nullptr;
    std::vector<sphgpu_material> materials;
    sphgpu_config config;

public:
    DeviceState(const RunSettings& settings, const Storage& storage, int precision);
    ~DeviceState();
    DeviceState(const DeviceState&) = delete;
    DeviceState& operator=(const DeviceState&) = delete;

    sphgpu_handle* get() const {
        return handle;
    }
    Size particleCount() const {
        return config.particle_count;
    }
    /// Throws InvalidSetup / Exception for a non-zero status.
    void check(int status) const;
    /// Copies every input quantity of the path from the storage to the device.
    void upload(const Storage& storage);
    /// Copies the state (values and derivatives) back into the storage.
    void download(Storage& storage, bool derivativesOnly) const;
};

/// ISolver drop-in: one ISolver::integrate evaluated on the GPU (materials initialize, gravity, pair
/// loop, finalize), same quantities as the reference solver.
class GpuSolver : public ISolver {
    RunSettings settings;
    int precision;
    mutable std::unique_ptr<DeviceState> device;

public:
    GpuSolver(IScheduler& scheduler, const RunSettings& settings, int precision = SPHGPU_PRECISION_FP64);
    ~GpuSolver() override;

    virtual void integrate(Storage& storage, Statistics& stats) override;
    virtual void create(Storage& storage, IMaterial& material) const override;

    /// Device state shared with GpuTimeStepping (created on first use).
    DeviceState& getDevice(const Storage& storage) const;
};

/// ISolver drop-in for HardSphereSolver (core/gravity/NBodySolver.h:24-140): Barnes-Hut self-gravity
/// (integrate) and the time-ordered collision loop with the configured handlers (collide) run on the GPU. The
/// host Storage is uploaded before and read back after each call; particles merged on the device are removed
/// from it with Storage::remove, as the reference solver does. Driven by the reference's own LeapFrog.
class GpuHardSphereSolver : public ISolver {
    RunSettings settings;
    int precision;
    sphgpu_handle* handle = nullptr;
    Size count = 0;
    uint64_t collisionTotals[4] = { 0, 0, 0, 0 };

    void ensure(const Storage& storage);
    void check(int status) const;
    void upload(const Storage& storage);
    void download(Storage& storage, bool positions);

public:
    GpuHardSphereSolver(IScheduler& scheduler, const RunSettings& settings, int precision = SPHGPU_PRECISION_FP64);
    ~GpuHardSphereSolver() override;

    virtual void integrate(Storage& storage, Statistics& stats) override;
    virtual void collide(Storage& storage, Statistics& stats, const Float dt) override;
    virtual void create(Storage& storage, IMaterial& material) const override;
};

/// When GpuTimeStepping copies the device state into the host Storage.
enum class SyncMode {
    EVERY_STEP, ///< after every step (every host consumer sees the current state)
    ON_DEMAND   ///< only in sync(): the device is the authoritative copy between outputs
};

/// ITimeStepping drop-in running the whole predictor-corrector (or leap-frog) step and the time-step
/// criteria on the device. The time step of ITimeStepping::step comes from the device (GpuCriterion), so the
/// host Storage needs no update between steps in ON_DEMAND mode; it is uploaded before the first step and
/// after invalidate() (a resumed run, host-side edits).
class GpuTimeStepping : public ITimeStepping {
public:
    struct Link {
        DeviceState* device = nullptr;
    };

private:
    std::shared_ptr<Link> link;
    SyncMode mode;
    bool uploaded = false;
    bool hostCurrent = true;

public:
    GpuTimeStepping(const SharedPtr<Storage>& storage, const RunSettings& settings,
        SyncMode mode = SyncMode::EVERY_STEP);

    /// Copies the device state into the host Storage if it is behind (ON_DEMAND mode).
    void sync();

    /// The host Storage was replaced or changed (BinaryInput::load of a resumed run, host-side edits):
    /// upload it before the next step.
    void invalidate();

    /// Number of device-to-host synchronisations so far.
    Size syncCount() const {
        return syncs;
    }

private:
    Size syncs = 0;

protected:
    virtual void stepParticles(IScheduler& scheduler, ISolver& solver, Statistics& stats) override;
};

/// IOutput decorator (e.g. around BinaryOutput, core/io/Output.cpp:481): synchronises the device state
/// into the host Storage, then lets the wrapped output write it. IRun::run calls dump only at output times
/// (core/run/IRun.cpp:251-256), so the device-to-host traffic happens at output times only.
class GpuOutput : public IOutput {
    AutoPtr<IOutput> output;
    GpuTimeStepping& stepping;

public:
    GpuOutput(AutoPtr<IOutput>&& output, GpuTimeStepping& stepping);

    virtual Expected<Path> dump(const Storage& storage, const Statistics& stats) override;
};

class GpuFinder;

/// IGravity drop-in: k-d tree, moments and tree walk on the device. getFinder returns a GpuFinder over the
/// positions of the last build (built on first use after each build), as BarnesHut returns its k-d tree
/// (core/gravity/BarnesHut.cpp:496-499).
class GpuBarnesHut : public IGravity {
    RunSettings settings;
    mutable std::unique_ptr<DeviceState> device;
    ArrayView<const Vector> positions;
    mutable std::unique_ptr<GpuFinder> finder;
    mutable bool finderCurrent = false;

public:
    explicit GpuBarnesHut(const RunSettings& settings);
    ~GpuBarnesHut() override;

    virtual void build(IScheduler& scheduler, const Storage& storage) override;
    virtual void evalSelfGravity(IScheduler& scheduler, ArrayView<Vector> dv, Statistics& stats) const override;
    virtual void evalAttractors(IScheduler& scheduler,
        ArrayView<Attractor> attractors,
        ArrayView<Vector> dv) const override;
    virtual Vector evalAcceleration(const Vector& r0) const override;
    virtual Float evalEnergy(IScheduler& scheduler, Statistics& stats) const override;
    virtual RawPtr<const IBasicFinder> getFinder() const override;
};

/// ISymmetricFinder drop-in on the library's cell grid. One device handle is kept across builds (created again
/// only when the particle count changes). The query of SymmetricSolver::loop, findAll / findLowerRank(i, 2 h_i),
/// is answered from the per-particle lists of sphgpu_get_radius_pairs fetched at build; every other query (another
/// radius, an arbitrary point) runs on the device (sphgpu_find_neighbors). The sets are those of KdTree::find.
class GpuFinder : public FinderTemplate<GpuFinder> {
    sphgpu_handle* handle = nullptr;
    Size handleCount = 0;
    std::vector<Size> start;
    std::vector<Size> neighbours;
    mutable std::vector<uint32_t> queryIdx;
    mutable std::vector<double> queryDistSqr;

protected:
    virtual void buildImpl(IScheduler& scheduler, ArrayView<const Vector> points) override;

public:
    explicit GpuFinder(const RunSettings& settings);
    ~GpuFinder() override;
    GpuFinder(const GpuFinder&) = delete;
    GpuFinder& operator=(const GpuFinder&) = delete;

    template <bool FindAll>
    Size find(const Vector& pos, const Size index, const Float radius, Array<NeighborRecord>& neighs) const;
};

} // namespace Gpu

NAMESPACE_SPH_END
