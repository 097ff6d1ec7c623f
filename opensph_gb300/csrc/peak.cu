// peak.cu — measured FP32 FMA rate of the device, the denominator of the FP32 roofline reports (the mixed
// Barnes-Hut walk is FP32-pipe bound). No counterpart in the reference.
//
// Every thread runs CHAINS independent FMA chains (enough in flight to cover the pipe latency) for a fixed number
// of iterations on every SM; the rate is 2 x CHAINS x iterations x threads / the CUDA-event time of the launch.

#include <algorithm>

#include "state.h"

namespace sphgpu {
namespace {

constexpr int PEAK_THREADS = 256;
constexpr int CHAINS = 8;

__global__ void __launch_bounds__(PEAK_THREADS) fmaChainKernel(uint32_t iterations, float b, float c, float* sink) {
    float a[CHAINS];
    for (int k = 0; k < CHAINS; ++k) {
        a[k] = float(threadIdx.x + k) * 1e-3f;
    }
    for (uint32_t it = 0; it < iterations; ++it) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
#pragma unroll
            for (int k = 0; k < CHAINS; ++k) {
                a[k] = fmaf(a[k], b, c);
            }
        }
    }
    float s = 0.f;
    for (int k = 0; k < CHAINS; ++k) {
        s += a[k];
    }
    // never true for the values used; keeps the chains live
    if (s == 1.2345678e30f) {
        sink[blockIdx.x * blockDim.x + threadIdx.x] = s;
    }
}

} // namespace
} // namespace sphgpu

extern "C" sphgpu_status sphgpu_measure_fp32_peak(double ms_target, double* tflops) {
    using namespace sphgpu;
    if (!tflops || !(ms_target > 0.)) {
        return SPHGPU_ERR_ARGUMENT;
    }
    int dev = 0, sms = 0, perSm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, fmaChainKernel, PEAK_THREADS, 0) != cudaSuccess) {
        return SPHGPU_ERR_CUDA;
    }
    const int blocks = std::max(1, sms * perSm);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    // warm-up, then one launch sized from the warm-up to about ms_target
    uint32_t iterations = 1024;
    float ms = 0.f;
    cudaError_t err = cudaSuccess;
    for (int round = 0; round < 3 && err == cudaSuccess; ++round) {
        cudaEventRecord(e0, 0);
        fmaChainKernel<<<blocks, PEAK_THREADS>>>(iterations, 0.999999f, 1e-7f, nullptr);
        cudaEventRecord(e1, 0);
        err = cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        if (round < 2 && ms > 0.f) {
            const double scale = ms_target / double(ms);
            iterations = uint32_t(std::min(1.0e9, std::max(1024.0, double(iterations) * scale)));
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (err != cudaSuccess || !(ms > 0.f)) {
        return SPHGPU_ERR_CUDA;
    }
    const double flops = 2.0 * CHAINS * 16.0 * double(iterations) * double(blocks) * PEAK_THREADS;
    *tflops = flops / (double(ms) * 1e-3) / 1e12;
    return SPHGPU_OK;
}
