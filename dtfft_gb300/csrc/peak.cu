// FP64 FMA throughput of this GPU, for the roofline of the complex128 and
// float64 transforms (their FFT kernels are bound by the FP64 pipe, not by
// HBM).  Each thread runs 8 independent FMA chains; the grid fills every SM.
#include <algorithm>

#include "common.cuh"
#include "dtfft_gb300.h"

namespace gb {

constexpr int kPeakChains = 8;
constexpr int kPeakIters = 4096;

__global__ void __launch_bounds__(256) fp64_fma_kernel(double* out, double b, double c) {
    double a[kPeakChains];
#pragma unroll
    for (int k = 0; k < kPeakChains; ++k) a[k] = threadIdx.x * 1e-9 + k;
    for (int it = 0; it < kPeakIters; ++it) {
#pragma unroll
        for (int k = 0; k < kPeakChains; ++k) a[k] = fma(a[k], b, c);
    }
    double s = 0;
#pragma unroll
    for (int k = 0; k < kPeakChains; ++k) s += a[k];
    // keeps the chains live; b and c make the sum stay tiny, so this never stores
    if (s == 123.456) out[blockIdx.x] = s;
}

}  // namespace gb

extern "C" int32_t dtfft_gb_measure_fp64_fma(double* tflops) {
    if (!tflops) return DTFFT_ERROR_INVALID_USAGE;
    int dev = 0, sms = 0;
    GB_CUDA_TRY(cudaGetDevice(&dev));
    GB_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    int per_sm = 0;
    GB_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gb::fp64_fma_kernel, 256, 0));
    const int blocks = sms * std::max(per_sm, 1) * 4;
    cudaEvent_t e0, e1;
    GB_CUDA_TRY(cudaEventCreate(&e0));
    GB_CUDA_TRY(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        cudaEventRecord(e0, 0);
        gb::fp64_fma_kernel<<<blocks, 256>>>(nullptr, 0.999999, 1e-12);
        cudaEventRecord(e1, 0);
        GB_CUDA_TRY(cudaEventSynchronize(e1));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    GB_CUDA_TRY(cudaGetLastError());
    const double flops = 2.0 * gb::kPeakChains * gb::kPeakIters * 256.0 * blocks;
    *tflops = flops / (best * 1e-3) / 1e12;
    return DTFFT_SUCCESS;
}
