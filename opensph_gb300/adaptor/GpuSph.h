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
/// Errors reported by the library are rethrown as the reference's InvalidSetup (configuration) or
/// Exception (runtime) types.

#include "gravity/IGravity.h"
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

/// ITimeStepping drop-in running the whole predictor-corrector (or leap-frog) step and the Courant
/// criterion on the device; the host storage is synchronised after each step.
class GpuTimeStepping : public ITimeStepping {
public:
    GpuTimeStepping(const SharedPtr<Storage>& storage, const RunSettings& settings);

protected:
    virtual void stepParticles(IScheduler& scheduler, ISolver& solver, Statistics& stats) override;
};

/// IGravity drop-in: k-d tree, moments and tree walk on the device.
class GpuBarnesHut : public IGravity {
    RunSettings settings;
    mutable std::unique_ptr<DeviceState> device;

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

/// ISymmetricFinder drop-in: the pair set of the GPU grid, answered per particle from CSR lists.
class GpuFinder : public FinderTemplate<GpuFinder> {
    std::vector<Size> start;
    std::vector<Size> neighbours;
    RunSettings settings;

protected:
    virtual void buildImpl(IScheduler& scheduler, ArrayView<const Vector> points) override;

public:
    explicit GpuFinder(const RunSettings& settings);

    template <bool FindAll>
    Size find(const Vector& pos, const Size index, const Float radius, Array<NeighborRecord>& neighs) const;
};

} // namespace Gpu

NAMESPACE_SPH_END
