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
// in srhd_mlp.cu. One CTA of kThreads threads evaluates kZones zones: each
// warp runs layer 2 for 32 zones as two 16-row tiles with mma.m16n8k16.
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

namespace mara {
namespace mlp {

constexpr int kIn = 4;
constexpr int kHidden = 64;
constexpr int kThreads = 128;
constexpr int kZones = 128;          // zones per CTA = 4 warps x 32
constexpr int kPad = 8;              // bf16 row padding (bank-conflict-free fragment loads)

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
    float w1[kHidden][kIn];
    float b1[kHidden], b2[kHidden], w3[kHidden];
    float norm_shift[kIn], norm_scale[kIn];
    float b3, out_shift, out_scale;
    __align__(16) __nv_bfloat16 w2[kHidden][kHidden + kPad];
    __align__(16) __nv_bfloat16 h1[kZones][kHidden + kPad];
    float feat[kZones][kIn];
    float out[kZones];
};

__device__ inline void load_weights(const Weights& w, Shared& s)
{
    for (int i = threadIdx.x; i < kHidden * kIn; i += blockDim.x) (&s.w1[0][0])[i] = (&w.w1[0][0])[i];
    for (int i = threadIdx.x; i < kHidden; i += blockDim.x)
    {
        s.b1[i] = w.b1[i];
        s.b2[i] = w.b2[i];
        s.w3[i] = w.w3[i];
    }
    for (int i = threadIdx.x; i < kHidden * kHidden; i += blockDim.x)
        s.w2[i / kHidden][i % kHidden] = w.w2_bf16[i / kHidden][i % kHidden];
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

__device__ inline uint32_t lds32(const __nv_bfloat16* p)
{
    return *reinterpret_cast<const uint32_t*>(p);
}

// D = A(16x16 bf16, row) * B(16x8 bf16, col) + C (f32)
__device__ inline void mma_bf16_16816(float c[4], const uint32_t a[4], const uint32_t b[2])
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Network forward for the kZones staged zones; result in s.out (the raw y).
__device__ inline void forward(Shared& s)
{
    // layer 1: one zone per thread
    for (int z = threadIdx.x; z < kZones; z += blockDim.x)
    {
        float x0 = s.feat[z][0], x1 = s.feat[z][1], x2 = s.feat[z][2], x3 = s.feat[z][3];
        for (int j = 0; j < kHidden; j += 2)
        {
            float h0 = s.b1[j] + s.w1[j][0] * x0 + s.w1[j][1] * x1 + s.w1[j][2] * x2 + s.w1[j][3] * x3;
            float h1 = s.b1[j + 1] + s.w1[j + 1][0] * x0 + s.w1[j + 1][1] * x1 + s.w1[j + 1][2] * x2 + s.w1[j + 1][3] * x3;
            *reinterpret_cast<__nv_bfloat162*>(&s.h1[z][j]) = __floats2bfloat162_rn(fast_tanh(h0), fast_tanh(h1));
        }
    }
    __syncthreads();

    // layer 2 + 3: warp w owns zones [32w, 32w + 32)
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    for (int mt = 0; mt < 2; ++mt)
    {
        const int row0 = warp * 32 + mt * 16 + g;
        float acc[8][4];
        for (int nt = 0; nt < 8; ++nt)
            for (int q = 0; q < 4; ++q) acc[nt][q] = 0.f;
        for (int ks = 0; ks < 4; ++ks)
        {
            const int k0 = ks * 16 + 2 * t;
            uint32_t a[4];
            a[0] = lds32(&s.h1[row0][k0]);
            a[1] = lds32(&s.h1[row0 + 8][k0]);
            a[2] = lds32(&s.h1[row0][k0 + 8]);
            a[3] = lds32(&s.h1[row0 + 8][k0 + 8]);
            for (int nt = 0; nt < 8; ++nt)
            {
                uint32_t b[2];
                b[0] = lds32(&s.w2[nt * 8 + g][k0]);
                b[1] = lds32(&s.w2[nt * 8 + g][k0 + 8]);
                mma_bf16_16816(acc[nt], a, b);
            }
        }
        // bias + tanh, then this thread's part of w3 . h2 for rows row0 and row0 + 8
        float y0 = 0.f, y1 = 0.f;
        for (int nt = 0; nt < 8; ++nt)
        {
            const int n0 = nt * 8 + 2 * t;
            y0 += s.w3[n0] * fast_tanh(acc[nt][0] + s.b2[n0]) + s.w3[n0 + 1] * fast_tanh(acc[nt][1] + s.b2[n0 + 1]);
            y1 += s.w3[n0] * fast_tanh(acc[nt][2] + s.b2[n0]) + s.w3[n0 + 1] * fast_tanh(acc[nt][3] + s.b2[n0 + 1]);
        }
        y0 += __shfl_xor_sync(0xffffffffu, y0, 1);
        y0 += __shfl_xor_sync(0xffffffffu, y0, 2);
        y1 += __shfl_xor_sync(0xffffffffu, y1, 1);
        y1 += __shfl_xor_sync(0xffffffffu, y1, 2);
        if (t == 0)
        {
            s.out[row0] = s.out_shift + s.out_scale * (y0 + s.b3);
            s.out[row0 + 8] = s.out_shift + s.out_scale * (y1 + s.b3);
        }
    }
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
