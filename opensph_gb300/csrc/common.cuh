// common.cuh — device-side helpers shared by the kernels of libsphgpu.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cfloat>

#include "../../include/sphgpu.h"

namespace sphgpu {

// a reference Vector {x, y, z, h}: 32-byte aligned so that one particle is one aligned 32-byte sector
using dbl4 = double4_32a;
__host__ __device__ __forceinline__ dbl4 mkd4(double x, double y, double z, double w) {
    return make_double4_32a(x, y, z, w);
}

// core/math/MathUtils.h:26-38: EPS and LARGE are float literals widened to double
#define SPH_EPS (double(1.e-12f))
#define SPH_LARGE (double(1.e20f))
#define SPH_PI 3.14159265358979323846264338327950288419716939937510

constexpr int LUT_ENTRIES = 40000; // core/sph/kernel/Kernel.h:53

// Device error word bits (read back by the host after a step; no trap, no assert on the device)
enum DeviceError : uint32_t {
    DEV_ERR_NODE_CAPACITY = 1u << 0,   // tree node pool exhausted
    DEV_ERR_WALK_CAPACITY = 1u << 1,   // tree-walk checklist overflow
    DEV_ERR_SEGMENT_CAPACITY = 1u << 2, // build work list overflow
    DEV_ERR_LEAF_SIZE = 1u << 3,       // leaf larger than a warp
    DEV_ERR_NONFINITE = 1u << 4,
    DEV_ERR_PAIR_CAPACITY = 1u << 5,
};

// Per-material constants kept in device memory (copied once from sphgpu_material)
struct MaterialD {
    int eos, yielding, damage, pad;
    double rho0, A, B, a, b, alpha, beta, u0, uiv, ucv, gamma;
    double mu, limit, u_melt, young;
    double rho_lo, rho_hi, u_lo, u_hi, d_lo, d_hi;
    double rho_min, u_min, s_min, d_min; // IMaterial::minimal (derivative time-step criterion)
    double inv_rho0, inv_u0, inv_u_melt;   // reciprocals (0 for a zero constant), for the mixed path's material update
};

// Uniform grid of the neighbour search (computed on the device each step)
// A fine grid (the mixed SPH step) has cells of about h_max: the pairs of a particle lie within span = 2 cells in each
// direction, and the mixed path's FP32 positions are relative to the origin of the coarse cell of 2 x 2 x 2 fine
// cells (fine coordinate >> shift). Otherwise the cells are at least 2 h_max, span = 1 and shift = 0.
struct GridInfo {
    double lo[3];      // grid origin
    double cell;       // cell edge
    double inv_cell;
    double hmax;
    int dims[3];
    uint32_t ncells;
    float lo_f[3];     // FP32 copy of the origin (mixed path)
    float pad;
    double ccell;      // coarse cell edge, cell << shift (origin of the mixed path's relative positions)
    int span;          // cells of the pair stencil on each side
    int shift;         // coarse coordinate = cell coordinate >> shift
};

struct Vec3 {
    double x, y, z;
};

__device__ __forceinline__ double sqr(double x) {
    return x * x;
}

// atomic min/max on non-negative doubles through their ordered bit patterns
__device__ __forceinline__ void atomicMinPos(double* addr, double v) {
    atomicMin(reinterpret_cast<unsigned long long*>(addr), static_cast<unsigned long long>(__double_as_longlong(v)));
}

// float <-> orderable uint32 (total order on finite floats, used by min/max reductions of positions)
__device__ __forceinline__ uint32_t floatFlip(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ unsigned long long doubleFlip(double f) {
    unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(f));
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double doubleUnflip(unsigned long long u) {
    u = (u & 0x8000000000000000ull) ? (u & 0x7fffffffffffffffull) : ~u;
    return __longlong_as_double(static_cast<long long>(u));
}

// Order key of a double that is not NaN: x < y <=> orderKey(x) < orderKey(y) and x == y <=> equal keys
// (-0 and +0 map to one key). Comparisons and minima on keys run on the integer pipe.
__device__ __forceinline__ unsigned long long orderKey(double f) {
    unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(f));
    if (u == 0x8000000000000000ull) {
        u = 0ull;
    }
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}

inline int ceilDiv(long long a, long long b) {
    return int((a + b - 1) / b);
}

} // namespace sphgpu
