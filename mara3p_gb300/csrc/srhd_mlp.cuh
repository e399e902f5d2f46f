// Learned pressure guess for SRHD primitive recovery: a 4-64-64-1 MLP.
//
// With E = tau + D, S = |S| and q = E^2 - S^2 - D^2 (computed in FP64: it is a
// small difference of large terms for fast, cold zones), the exact pressure
// satisfies p*E/q in [1/6, 1/3] for gamma = 4/3 (q = 6 p rho W^2 + 8 p^2 W^2
// + p^2), so the network learns y = log(p E / q), a smooth O(1) correction:
//   features  x = normalised (log(q/E^2), S/E, D/E, log((E - S)/E))
//   layer 1   h1 = tanh(W1 x + b1)        FP32 on the CUDA cores (K = 4)
//   layer 2   h2 = tanh(W2 h1 + b2)       BF16 operands, FP32 accumulate, tensor cores
//   layer 3   y  = w3 . h2 + b3           FP32
//   guess     p  = exp(out_shift + out_scale * y) * q / E
//
// Weights live in one device struct (Weights) written by the training kernels
// in srhd_mlp.cu. One CTA of kThreads threads evaluates kZones = 128 zones.
// Layer 2 is one 128 x 64 x 64 tcgen05 MMA chain (kind::f16, BF16 operands in
// shared memory, FP32 accumulator in 64 columns of tensor memory): the
// activations h1 (A, 128 x 64) and W2 (B, 64 x 64) are stored K-major in the
// no-swizzle core-matrix layout (8 rows x 16 bytes per core matrix; leading
// byte offset = the stride between core matrices along K, stride byte offset
// = the stride between 8-row groups), one thread issues the four K = 16 steps
// and commits them to an mbarrier, and each warp reads its 32 rows back with
// tcgen05.ld (lane = zone, column = hidden unit).
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

namespace mara {
namespace mlp {

constexpr int kIn = 4;
constexpr int kHidden = 64;
constexpr int kThreads = 128;        // one zone per thread in layers 2-3: kThreads == kZones
constexpr int kZones = 128;          // zones per CTA = 4 warps x 32
constexpr int kTmemColumns = 64;     // FP32 accumulator columns of layer 2 (one per hidden unit)
// core-matrix layout strides (bytes): along K, 8-row group to 8-row group
constexpr uint32_t kCoreBytes = 128;
constexpr uint32_t kAKStride = (kZones / 8) * kCoreBytes;     // 2048
constexpr uint32_t kBKStride = (kHidden / 8) * kCoreBytes;    // 1024
constexpr uint32_t kABytes = kZones * kHidden * 2, kBBytes = kHidden * kHidden * 2;
// bounded wait for the MMA's mbarrier (tries of mbarrier.try_wait)
constexpr int kWaitTries = 1 << 22;
static_assert(kThreads == 128 && kZones == 128, "the layer-2 epilogue maps 4 warps onto the 128 TMEM lanes");

struct Weights
{
    float norm_shift[kIn], norm_scale[kIn];
    float w1[kHidden][kIn];          // [out][in]
    float b1[kHidden];
    float w2[kHidden][kHidden];      // FP32 master, [out n][in k]
    float b2[kHidden];
    float w3[kHidden];
    float b3;
    float out_shift, out_scale;
    __nv_bfloat16 w2_bf16[kHidden][kHidden];   // [n][k], BF16 copy used by inference
};

struct Shared
{
    __align__(128) unsigned char a[kABytes];    // h1, core-matrix layout (16 KB)
    __align__(128) unsigned char b[kBBytes];    // W2 (BF16), core-matrix layout (8 KB)
    float w1[kHidden][kIn];
    float b1[kHidden], b2[kHidden], w3[kHidden];
    float norm_shift[kIn], norm_scale[kIn];
    float b3, out_shift, out_scale;
    float feat[kZones][kIn];
    float out[kZones];
    __align__(8) unsigned long long mbar;
    uint32_t tmem;
};

// byte offset of element (row, k) of a K-major operand with kstride bytes between K core matrices
__device__ inline uint32_t core_offset(int row, int k, uint32_t kstride)
{
    return uint32_t(row >> 3) * kCoreBytes + uint32_t(k >> 3) * kstride + uint32_t(row & 7) * 16u + uint32_t(k & 7) * 2u;
}

__device__ inline uint32_t smem_addr(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }

// tcgen05 shared-memory matrix descriptor, no swizzle
__device__ inline uint64_t matrix_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return uint64_t((addr >> 4) & 0x3FFFu) | (uint64_t((lbo >> 4) & 0x3FFFu) << 16) |
           (uint64_t((sbo >> 4) & 0x3FFFu) << 32) | (uint64_t(1) << 46);
}

// Copy the weights into shared memory (W2 into the MMA's B layout), allocate
// the CTA's tensor memory (warp 0) and initialise the MMA barrier. Every
// thread of the CTA calls it once, before any forward; end() releases.
__device__ inline void begin(const Weights& w, Shared& s)
{
    if (threadIdx.x < 32)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_addr(&s.tmem)), "r"(kTmemColumns));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (threadIdx.x == 0)
    {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_addr(&s.mbar)), "r"(1));
        asm volatile("fence.mbarrier_init.release.cluster;");
    }
    for (int i = threadIdx.x; i < kHidden * kIn; i += blockDim.x) (&s.w1[0][0])[i] = (&w.w1[0][0])[i];
    for (int i = threadIdx.x; i < kHidden; i += blockDim.x)
    {
        s.b1[i] = w.b1[i];
        s.b2[i] = w.b2[i];
        s.w3[i] = w.w3[i];
    }
    // W2 rows are only 4-byte aligned inside Weights: read four words, store one 16-byte core row
    for (int i = threadIdx.x; i < kHidden * kHidden / 8; i += blockDim.x)
    {
        const int n = i / (kHidden / 8), k = (i % (kHidden / 8)) * 8;
        const uint32_t* src = reinterpret_cast<const uint32_t*>(&w.w2_bf16[n][k]);
        *reinterpret_cast<uint4*>(s.b + core_offset(n, k, kBKStride)) = make_uint4(src[0], src[1], src[2], src[3]);
    }
    if (threadIdx.x < kIn)
    {
        s.norm_shift[threadIdx.x] = w.norm_shift[threadIdx.x];
        s.norm_scale[threadIdx.x] = w.norm_scale[threadIdx.x];
    }
    if (threadIdx.x == 0)
    {
        s.b3 = w.b3;
        s.out_shift = w.out_shift;
        s.out_scale = w.out_scale;
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
}

// Release the tensor memory (after the last forward; every thread calls it).
__device__ inline void end(Shared& s)
{
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    if (threadIdx.x < 32)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(s.tmem), "r"(kTmemColumns));
}

// E = tau + D and q = E^2 - S^2 - D^2 of one zone, in FP64.
__host__ __device__ inline void zone_invariants(double D, double S1, double S2, double S3, double tau,
                                                double& E, double& q, double& SS)
{
    E = tau + D;
    SS = S1 * S1 + S2 * S2 + S3 * S3;
    q = (E - D) * (E + D) - SS;
}

// Raw (un-normalised) features of one zone; false if the zone has no
// physical solution (q <= 0 or E <= 0), in which case no guess is made.
__host__ __device__ inline bool raw_features(double D, double S1, double S2, double S3, double tau, float f[4])
{
    double E, q, SS;
    zone_invariants(D, S1, S2, S3, tau, E, q, SS);
    if (!(q > 0.0) || !(E > 0.0) || !(D > 0.0))
    {
        f[0] = f[1] = f[2] = f[3] = 0.0f;
        return false;
    }
    float Ef = float(E), S = sqrtf(float(SS));
    f[0] = logf(float(q / (E * E)));
    f[1] = S / Ef;
    f[2] = float(D) / Ef;
    f[3] = logf(float(q + D * D) / ((Ef + S) * Ef));
    return true;
}

__device__ inline bool features(double D, double S1, double S2, double S3, double tau, float f[4])
{
    return raw_features(D, S1, S2, S3, tau, f);
}

__device__ inline void stage_features(Shared& s, int zone, const float f[4])
{
    for (int k = 0; k < kIn; ++k) s.feat[zone][k] = (f[k] - s.norm_shift[k]) * s.norm_scale[k];
}

__device__ inline float fast_tanh(float x)
{
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Network forward for the kZones staged zones; result in s.out (the raw y, or
// -infinity, which maps to the reference's start p = 0, if the MMA did not
// complete within the wait bound). phase: the barrier phase this CTA waits on
// next (0 for the first forward); every thread of the CTA calls forward.
__device__ inline void forward(Shared& s, uint32_t& phase)
{
    // layer 1: one zone per thread, 8 hidden units per 16-byte store into the A layout
    for (int z = threadIdx.x; z < kZones; z += blockDim.x)
    {
        const float x0 = s.feat[z][0], x1 = s.feat[z][1], x2 = s.feat[z][2], x3 = s.feat[z][3];
        for (int j = 0; j < kHidden; j += 8)
        {
            uint32_t packed[4];
            for (int q = 0; q < 4; ++q)
            {
                const int a = j + 2 * q, b = a + 1;
                const float h0 = s.b1[a] + s.w1[a][0] * x0 + s.w1[a][1] * x1 + s.w1[a][2] * x2 + s.w1[a][3] * x3;
                const float h1 = s.b1[b] + s.w1[b][0] * x0 + s.w1[b][1] * x1 + s.w1[b][2] * x2 + s.w1[b][3] * x3;
                const __nv_bfloat162 v = __floats2bfloat162_rn(fast_tanh(h0), fast_tanh(h1));
                packed[q] = *reinterpret_cast<const uint32_t*>(&v);
            }
            *reinterpret_cast<uint4*>(s.a + core_offset(z, j, kAKStride)) = make_uint4(packed[0], packed[1], packed[2], packed[3]);
        }
    }
    // the generic-proxy stores must be visible to the tensor cores' reads
    asm volatile("fence.proxy.async.shared::cta;");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");

    // layer 2: D[128 x 64] = h1[128 x 64] W2^T, four K = 16 steps, one thread issues
    if (threadIdx.x == 0)
    {
        const uint32_t idesc = (1u << 4)                         // D: FP32
                             | (1u << 7) | (1u << 10)            // A, B: BF16 (both K-major)
                             | (uint32_t(kHidden >> 3) << 17)    // N = 64
                             | (uint32_t(kZones >> 4) << 24);    // M = 128
        for (int ks = 0; ks < kHidden / 16; ++ks)
        {
            const uint64_t ad = matrix_desc(smem_addr(s.a) + ks * 2 * kAKStride, kAKStride, kCoreBytes);
            const uint64_t bd = matrix_desc(smem_addr(s.b) + ks * 2 * kBKStride, kBKStride, kCoreBytes);
            asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                         "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                         :: "r"(s.tmem), "l"(ad), "l"(bd), "r"(idesc), "r"(ks));
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                     :: "r"(smem_addr(&s.mbar)));
    }
    uint32_t done = 0;
    for (int it = 0; it < kWaitTries && !done; ++it)
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done) : "r"(smem_addr(&s.mbar)), "r"(phase));
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;");

    // layers 2 (bias, tanh) and 3: warp w holds rows 32w .. 32w + 31, one zone per thread
    const int warp = threadIdx.x >> 5, row = threadIdx.x;
    uint32_t r[64];
    const uint32_t taddr = s.tmem + (uint32_t(warp * 32) << 16);
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32, %33, %34, %35, %36, %37, %38, %39, %40, %41, %42, %43, %44, %45, %46, %47, %48, %49, %50, %51, %52, %53, %54, %55, %56, %57, %58, %59, %60, %61, %62, %63}, [%64];" : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63]) : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;");
    float y = 0.0f;
    for (int n = 0; n < kHidden; ++n) y += s.w3[n] * fast_tanh(__uint_as_float(r[n]) + s.b2[n]);
    s.out[row] = done ? s.out_shift + s.out_scale * (y + s.b3) : -__int_as_float(0x7f800000);
    asm volatile("tcgen05.fence::before_thread_sync;");
}

// Pressure guess from the network output; 0 (the reference's start) when the
// zone has no physical solution.
__device__ inline double pressure_from_output(float y, double D, double S1, double S2, double S3, double tau)
{
    double E, q, SS;
    zone_invariants(D, S1, S2, S3, tau, E, q, SS);
    if (!(q > 0.0) || !(E > 0.0)) return 0.0;
    return double(__expf(y)) * (q / E);
}

} // namespace mlp
} // namespace mara
