"""GB300-native (sm_103a) implementation of OpenSPH's per-step SPH + Barnes-Hut gravity hot path.

The compute lives in libsphgpu.so (CUDA C++, C ABI declared in include/sphgpu.h). This package holds the
ctypes binding (`abi`), the host-side mirror of the reference's solver / time-stepping interface
(`solver.GpuSolver`) and the build script (`build`).
"""
from . import abi  # noqa: F401

__all__ = ["abi"]
