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
    ScopedEvents events;
    MARA_CUDA(events.create(2));
    cudaEvent_t e0 = events[0], e1 = events[1];
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
    if (rc != MARA_OK) return rc;
    MARA_REQUIRE(best > 0.0f, "mara_measure_fp64_rate: timing failed");
    const double fmas = double(blocks) * kThreads * kChains * kIters;
    *dfma_per_second = fmas / (double(best) * 1e-3);
    return MARA_OK;
}

// ---------------------------------------------------------------- host link
// The rates of the host link in the forms the host-buffer calls use: copy
// engine both ways, and kernels reading and writing pinned host memory
// through its device address (16-byte accesses), alone and both at once.
namespace {

__global__ void link_copy_kernel(const double2* __restrict__ src, double2* __restrict__ dst, size_t n)
{
    for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
        dst[i] = src[i];
}

} // namespace

extern "C" int mara_measure_host_link(void* host, void* device, int64_t bytes, double* gbs, void* stream)
{
    using namespace mara;
    MARA_REQUIRE(host && device && gbs, "mara_measure_host_link: null buffer");
    MARA_REQUIRE(bytes >= (1 << 20) && bytes % 32 == 0, "mara_measure_host_link: bytes must be a multiple of 32, >= 1 MiB");
    cudaPointerAttributes pa;
    MARA_CUDA(cudaPointerGetAttributes(&pa, host));
    MARA_REQUIRE(pa.type == cudaMemoryTypeHost && pa.devicePointer, "mara_measure_host_link: host is not pinned host memory");
    MARA_REQUIRE((reinterpret_cast<uintptr_t>(pa.devicePointer) & 15) == 0 && (reinterpret_cast<uintptr_t>(device) & 15) == 0,
                 "mara_measure_host_link: buffers must be 16-byte aligned");
    cudaStream_t s = as_stream(stream);
    int dev = 0, sms = 0;
    MARA_CUDA(cudaGetDevice(&dev));
    MARA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * 16;
    auto* hdev = static_cast<double2*>(pa.devicePointer);
    auto* d = static_cast<double2*>(device);
    const size_t n = size_t(bytes) / 16, half = n / 2;
    cudaStream_t s2 = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr;
    MARA_CUDA(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking));
    int rc = cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess &&
             cudaEventCreate(&e2) == cudaSuccess ? MARA_OK : fail(MARA_ERR_CUDA, "mara_measure_host_link: event create");
    // best of three per form (after one untimed round), milliseconds
    double best[5] = {1e30, 1e30, 1e30, 1e30, 1e30};
    for (int rep = 0; rep < 4 && rc == MARA_OK; ++rep)
    {
        for (int form = 0; form < 5 && rc == MARA_OK; ++form)
        {
            cudaEventRecord(e0, s);
            if (form == 0) cudaMemcpyAsync(device, host, size_t(bytes), cudaMemcpyHostToDevice, s);
            else if (form == 1) cudaMemcpyAsync(host, device, size_t(bytes), cudaMemcpyDeviceToHost, s);
            else if (form == 2) link_copy_kernel<<<blocks, 256, 0, s>>>(hdev, d, n);
            else if (form == 3) link_copy_kernel<<<blocks, 256, 0, s>>>(d, hdev, n);
            else
            {
                // read one half of the host buffer while writing the other
                cudaStreamWaitEvent(s2, e0, 0);
                link_copy_kernel<<<blocks / 2, 256, 0, s>>>(hdev, d, half);
                link_copy_kernel<<<blocks / 2, 256, 0, s2>>>(d + half, hdev + half, n - half);
                cudaEventRecord(e2, s2);
                cudaStreamWaitEvent(s, e2, 0);
            }
            cudaEventRecord(e1, s);
            rc = launch_status("mara_measure_host_link");
            if (rc == MARA_OK && cudaEventSynchronize(e1) != cudaSuccess) rc = fail(MARA_ERR_CUDA, "mara_measure_host_link: sync");
            float ms = 0.0f;
            if (rc == MARA_OK && rep > 0 && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess && ms < best[form]) best[form] = ms;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);
    cudaStreamDestroy(s2);
    if (rc != MARA_OK) return rc;
    for (int f = 0; f < 5; ++f) gbs[f] = double(bytes) / (best[f] * 1e-3) / 1e9;
    return MARA_OK;
}
