// noalloc.cu — conserved totals without any allocation.
//
// Some callers of this library cannot call cudaMalloc: a host application that owns the whole device
// memory budget and hands out only pre-allocated buffers, or a per-step diagnostic hook that must not
// trigger the implicit device synchronisation a cudaMalloc / cudaFree may cause. For them this file
// provides sphgpu_totals_noalloc, a variant of the totals reduction behind sphgpu_totals whose scratch (one
// row of partial sums per block) lives in a file-scope __device__ array instead of a handle's allocation.
//
// Lifetime and sharing: the array is part of the library image, so every GPU that loads the library holds
// it (kTotalsScratchBytes, 72 KiB) until the process exits. All calls share it: two calls whose kernels
// overlap on the GPU (different streams, or different host threads) race on it and must be serialised by
// the caller. Each call writes every row it later reads, so nothing carries over from the previous call.
//
// Set-up: host code cannot use the array's name as a device address (on the host it names a stand-in
// object). Every call looks the address up with cudaGetSymbolAddress for the current device and context: a
// host-side query that queues no work, so the address is never stale (a cudaDeviceReset or another context
// loads the library image at a different address). The first call on a device may load the library's
// device code; make it before any stream capture begins.

#include "state.h"

namespace sphgpu {
namespace {

constexpr uint32_t kTotalsChunk = 4096;     // particles per block
constexpr uint32_t kTotalsMaxBlocks = 1024; // rows of the scratch array
constexpr uint32_t kTotalsThreads = 256;

static __device__ __align__(256) double gTotalsScratch[kTotalsMaxBlocks * 9];

__device__ __forceinline__ void neumaier(double& sum, double& c, double x) {
    const double t = sum + x;
    if (fabs(sum) >= fabs(x)) {
        c += (sum - t) + x;
    } else {
        c += (x - t) + sum;
    }
    sum = t;
}

// Block b sums particles [b * kTotalsChunk, (b + 1) * kTotalsChunk) into row b of the scratch.
__global__ void __launch_bounds__(kTotalsThreads) totalsPartialKernel(const double* __restrict__ r,
    const double* __restrict__ v, const double* __restrict__ m, const double* __restrict__ u, uint32_t n,
    double* scratch) {
    double sum[9], comp[9];
    for (int k = 0; k < 9; ++k) {
        sum[k] = 0.;
        comp[k] = 0.;
    }
    const uint32_t begin = blockIdx.x * kTotalsChunk;
    const uint32_t end = min(n, begin + kTotalsChunk);
    for (uint32_t i = begin + threadIdx.x; i < end; i += kTotalsThreads) {
        const double rx = r[4 * i], ry = r[4 * i + 1], rz = r[4 * i + 2];
        const double vx = v[4 * i], vy = v[4 * i + 1], vz = v[4 * i + 2];
        const double mi = m[i];
        neumaier(sum[0], comp[0], mi * vx);
        neumaier(sum[1], comp[1], mi * vy);
        neumaier(sum[2], comp[2], mi * vz);
        neumaier(sum[3], comp[3], mi * (ry * vz - rz * vy));
        neumaier(sum[4], comp[4], mi * (rz * vx - rx * vz));
        neumaier(sum[5], comp[5], mi * (rx * vy - ry * vx));
        neumaier(sum[6], comp[6], 0.5 * mi * (vx * vx + vy * vy + vz * vz));
        neumaier(sum[7], comp[7], mi * u[i]);
        neumaier(sum[8], comp[8], mi);
    }
    __shared__ double sh[9][kTotalsThreads];
    for (int k = 0; k < 9; ++k) {
        sh[k][threadIdx.x] = sum[k] + comp[k];
    }
    __syncthreads();
    if (threadIdx.x < 9) {
        double acc = 0., c = 0.;
        for (uint32_t t = 0; t < kTotalsThreads; ++t) {
            neumaier(acc, c, sh[threadIdx.x][t]);
        }
        scratch[blockIdx.x * 9 + threadIdx.x] = acc + c;
    }
}

// Adds the rows written by this call, in row order (deterministic for a given n).
__global__ void totalsFinalKernel(const double* __restrict__ scratch, uint32_t rows, double* out) {
    if (threadIdx.x < 9) {
        double acc = 0., c = 0.;
        for (uint32_t b = 0; b < rows; ++b) {
            neumaier(acc, c, scratch[b * 9 + threadIdx.x]);
        }
        out[threadIdx.x] = acc + c;
    }
}

} // namespace
} // namespace sphgpu

extern "C" sphgpu_status sphgpu_totals_noalloc(const double* r, const double* v, const double* m, const double* u,
    uint64_t n, double* totals, void* stream) {
    using namespace sphgpu;
    if (!r || !v || !m || !u || !totals) {
        return SPHGPU_ERR_ARGUMENT;
    }
    if (n > uint64_t(SPHGPU_TOTALS_NOALLOC_MAX_PARTICLES)) {
        // the scratch array holds one row per kTotalsChunk particles: larger sets need sphgpu_totals
        return SPHGPU_ERR_CAPACITY;
    }
    void* address = nullptr;
    if (cudaGetSymbolAddress(&address, gTotalsScratch) != cudaSuccess || !address) {
        return SPHGPU_ERR_CUDA;
    }
    double* scratch = static_cast<double*>(address);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const uint32_t rows = uint32_t((n + kTotalsChunk - 1) / kTotalsChunk);
    if (rows > 0) {
        totalsPartialKernel<<<rows, kTotalsThreads, 0, st>>>(r, v, m, u, uint32_t(n), scratch);
    }
    totalsFinalKernel<<<1, 32, 0, st>>>(scratch, rows, totals);
    return cudaGetLastError() == cudaSuccess ? SPHGPU_OK : SPHGPU_ERR_CUDA;
}
