// Measurement helper: the FP64 fused multiply-add rate of the current GPU,
// the roofline denominator of the kernels that the FP64 pipe bounds (the
// plain FP64 minidisk stage, the SRHD Newton recoveries, the sedov tracks).
// GB300 runs FP64 at a small fraction of its FP32 rate, so these kernels are
// compared with this rate rather than with HBM bandwidth.
#include <cuda_runtime.h>
#include "common.cuh"

namespace {

constexpr int kChains = 8;        // independent FMA chains per thread
constexpr int kIters = 1024;      // FMAs per chain
constexpr int kThreads = 256;

// keeps the chains' results live; every thread adds its own sum, so the value
// is meaningless but the FMAs cannot be removed
__device__ double g_fp64_sink;

__global__ void __launch_bounds__(kThreads) fma_rate_kernel(double a, double b, int write)
{
    double x[kChains];
    for (int c = 0; c < kChains; ++c) x[c] = double(threadIdx.x + c) * 1e-3;
    for (int it = 0; it < kIters; ++it)
    {
#pragma unroll
        for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
    }
    double s = 0.0;
    for (int c = 0; c < kChains; ++c) s += x[c];
    if (write) g_fp64_sink = s;   // never true at run time; the branch keeps s live
}

} // namespace

extern "C" int mara_measure_fp64_rate(double* dfma_per_second, void* stream)
{
    using namespace mara;
    MARA_REQUIRE(dfma_per_second != nullptr, "mara_measure_fp64_rate: null output");
    cudaStream_t s = as_stream(stream);
    int dev = 0, sms = 0, per_sm = 0;
    MARA_CUDA(cudaGetDevice(&dev));
    MARA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    MARA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fma_rate_kernel, kThreads, 0));
    const int blocks = sms * (per_sm > 0 ? per_sm : 1) * 4;
    cudaEvent_t e0, e1;
    MARA_CUDA(cudaEventCreate(&e0));
    MARA_CUDA(cudaEventCreate(&e1));
    float best = 0.0f;
    int rc = MARA_OK;
    for (int rep = 0; rep < 4 && rc == MARA_OK; ++rep)
    {
        // a = 1 - 2^-20, b = 2^-30: the chains stay finite and normal
        cudaEventRecord(e0, s);
        fma_rate_kernel<<<blocks, kThreads, 0, s>>>(1.0 - 0x1p-20, 0x1p-30, 0);
        cudaEventRecord(e1, s);
        rc = launch_status("fma_rate_kernel");
        if (rc == MARA_OK && cudaEventSynchronize(e1) == cudaSuccess)
        {
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep > 0 && (best == 0.0f || ms < best)) best = ms;   // the first launch is a warm-up
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != MARA_OK) return rc;
    MARA_REQUIRE(best > 0.0f, "mara_measure_fp64_rate: timing failed");
    const double fmas = double(blocks) * kThreads * kChains * kIters;
    *dfma_per_second = fmas / (double(best) * 1e-3);
    return MARA_OK;
}
