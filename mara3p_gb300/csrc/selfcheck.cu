// Self-check of the integer float <-> double conversions that the mixed
// kernels use in place of the FP64 pipe's (mixed_math.cuh), against the
// hardware conversions, on the device that runs them:
//   [0] f2d(x) for all 2^32 floats: the exact double of every normal float
//       and infinity, a NaN for every NaN, and the signed zero of x's sign
//       for every zero and subnormal;
//   [1] f2d_sum(x) for all 2^32 floats: as f2d for normal floats,
//       infinities and NaN; for zeros and subnormals a double of x's sign
//       below 2^-126 in magnitude;
//   [2] d2f(x) for 2^32 doubles whose high word runs over all 2^32 patterns
//       (sign, exponent and the top 20 mantissa bits) and whose low word is
//       a hash of it (every 16th an exact tie): round to nearest with ties
//       away from zero between 2^-126 and 2^128, the signed zero below
//       2^-126, and NaN at 2^128 and above, for infinities and for NaN.
#include <cuda_runtime.h>
#include "common.cuh"
#include "mixed_math.cuh"

namespace {

__device__ unsigned long long g_conversion_mismatches[3];

__device__ inline bool same_sign(double a, float x) { return (__double_as_longlong(a) < 0) == (__float_as_int(x) < 0); }

__device__ inline unsigned f2d_mismatch(unsigned u)
{
    const float x = __uint_as_float(u);
    const unsigned mag = u & 0x7FFFFFFFu;
    const double a = mara::f2d(x);
    if (mag > 0x7F800000u) return isnan(a) ? 0u : 1u;
    if (mag < 0x00800000u) return (a == 0.0 && same_sign(a, x)) ? 0u : 1u;
    return __double_as_longlong(a) == __double_as_longlong(double(x)) ? 0u : 1u;
}

__device__ inline unsigned f2d_sum_mismatch(unsigned u)
{
    const float x = __uint_as_float(u);
    const unsigned mag = u & 0x7FFFFFFFu;
    const double a = mara::f2d_sum(x);
    if (mag > 0x7F800000u) return isnan(a) ? 0u : 1u;
    if (mag < 0x00800000u) return (fabs(a) < 0x1p-126 && same_sign(a, x)) ? 0u : 1u;
    return __double_as_longlong(a) == __double_as_longlong(double(x)) ? 0u : 1u;
}

__device__ inline unsigned d2f_mismatch(unsigned u)
{
    unsigned lo = u * 0x9E3779B9u;
    lo ^= lo >> 15;
    lo *= 0x85EBCA6Bu;
    lo ^= lo >> 13;
    if ((u & 15u) == 0u) lo = (lo & 0xE0000000u) | 0x10000000u;   // every 16th: an exact tie
    const double x = __hiloint2double(int(u), int(lo));
    const float f = mara::d2f(x);
    const double ax = fabs(x);
    if (!(ax < 0x1p128)) return isnan(f) ? 0u : 1u;   // also infinities and NaN
    if (ax < 0x1p-126) return (f == 0.0f && (__float_as_int(f) < 0) == (u >> 31 != 0u)) ? 0u : 1u;
    // a tie sits exactly halfway between two floats: the 29 bits rounded
    // off are 1 followed by 28 zeros
    const bool tie = (lo & 0x1FFFFFFFu) == 0x10000000u;
    float expect = __double2float_rn(x);
    if (tie)
    {
        const float down = __double2float_rz(x);   // toward zero; away is one unit further
        expect = __uint_as_float(__float_as_uint(down) + 1u);
    }
    return __float_as_uint(f) == __float_as_uint(expect) ? 0u : 1u;
}

__global__ void __launch_bounds__(256) conversion_check_kernel()
{
    unsigned long long bad[3] = {0ull, 0ull, 0ull};
    const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * blockDim.x;
    for (unsigned long long i = static_cast<unsigned long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < (1ull << 32);
         i += stride)
    {
        const unsigned u = unsigned(i);
        bad[0] += f2d_mismatch(u);
        bad[1] += f2d_sum_mismatch(u);
        bad[2] += d2f_mismatch(u);
    }
    for (int k = 0; k < 3; ++k)
    {
        unsigned long long v = bad[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0 && v != 0ull) atomicAdd(&g_conversion_mismatches[k], v);
    }
}

} // namespace

extern "C" int mara_check_conversions(unsigned long long* mismatches, void* stream)
{
    using namespace mara;
    MARA_REQUIRE(mismatches != nullptr, "mara_check_conversions: null output");
    cudaStream_t s = as_stream(stream);
    void* counters = nullptr;
    MARA_CUDA(cudaGetSymbolAddress(&counters, g_conversion_mismatches));
    MARA_CUDA(cudaMemsetAsync(counters, 0, sizeof(unsigned long long) * 3, s));
    int dev = 0, sms = 0;
    MARA_CUDA(cudaGetDevice(&dev));
    MARA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    conversion_check_kernel<<<sms * 8, 256, 0, s>>>();
    if (int r = launch_status("conversion_check_kernel")) return r;
    MARA_CUDA(cudaMemcpyAsync(mismatches, counters, sizeof(unsigned long long) * 3, cudaMemcpyDeviceToHost, s));
    MARA_CUDA(cudaStreamSynchronize(s));
    return MARA_OK;
}
