// Arithmetic shared by the mixed-precision kernels: double <-> float
// conversions in integer instructions (GB300 runs FP64, conversions included,
// at a small fraction of the FP32 rate) and single-MUFU FP32 approximations.
#pragma once
#include <cuda_runtime.h>

namespace mara {

// double -> float and float -> double (exact) with integer instructions
// only, so that the mixed path issues no FP64-pipe work for them.
// d2f rounds to nearest with ties away from zero. For a double of biased
// exponent e = 896 + ef in the float range, bits 28..0 of the 64-bit pattern
// shifted left by 3 are e[7:0] and the top 23 mantissa bits, and e[7:0] is
// ef with bit 7 flipped; bit 28 of the low word is the first bit rounded off
// (a carry out of the mantissa correctly bumps the exponent). Magnitudes below
// the smallest normal float (1.2e-38) become signed zero; magnitudes of 2^128
// and beyond, infinities and NaNs become NaN.
__device__ inline float d2f(double x)
{
    const unsigned long long b = __double_as_longlong(x);
    const unsigned hi = unsigned(b >> 32), lo = unsigned(b);
    const unsigned sign = hi & 0x80000000u, mag = hi & 0x7FFFFFFFu;
    unsigned f = ((__funnelshift_l(lo, hi, 3) & 0x7FFFFFFFu) ^ 0x40000000u) + ((lo >> 28) & 1u);
    f = mag < 0x38100000u ? 0u : f;
    f = mag >= 0x47F00000u ? 0x7FC00000u : f;
    return __uint_as_float(f | sign);
}

// f2d: the magnitude bits shifted into place with the exponent rebiased by
// (1023 - 127) << 20, or by (2047 - 255) << 20 for infinities and NaN (whose
// payload moves with them); zero and subnormals become signed zero. Equal,
// for every one of the 2^32 inputs, to the field-by-field form it replaces.
__device__ inline double f2d(float x)
{
    const unsigned b = __float_as_uint(x);
    const unsigned mag = b & 0x7FFFFFFFu, sign = b & 0x80000000u;
    const unsigned bias = mag >= 0x7F800000u ? 0x70000000u : 0x38000000u;
    const bool tiny = mag < 0x00800000u;
    const unsigned hi = tiny ? sign : (((mag >> 3) + bias) | sign);
    const unsigned lo = tiny ? 0u : (b << 29);
    return __hiloint2double(int(hi), int(lo));
}

// f2d for an FP32 increment that is added to an FP64 state (u + x, or
// fma(x, h, u) with h = 1 or 1/2): the same double as f2d for every normal
// float, infinity and NaN (mara_check_conversions compares both with the
// hardware conversion over all 2^32 floats). Zeros and subnormals become
// doubles of the same sign below 2^-126 in magnitude, which the sum absorbs
// exactly wherever |u| >= 2^-72 (elsewhere it moves u by less than 2^-126).
// No zero test, and the infinity/NaN test is one FP32 comparison; the sign
// bit, shifted down three places with the rest, is masked back to bit 31.
__device__ __forceinline__ double f2d_sum(float x)
{
    const unsigned b = __float_as_uint(x);
    const bool special = !(fabsf(x) < __int_as_float(0x7F800000));
    const unsigned hi = (unsigned(int(b) >> 3) & 0x8FFFFFFFu) + (special ? 0x70000000u : 0x38000000u);
    return __hiloint2double(int(hi), int(b << 29));
}

// Single-MUFU approximations for the mixed path (relative error ~1e-7,
// well inside the FP32 budget of the fluxes; denormals flush to zero).
__device__ inline float rcp_fast(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// a / b from r = rcp_fast(b) and one correction by the exact residual
// a - b q0 (an FMA): q0 + r (a - b q0) is the correctly rounded quotient but
// in rare cases, and within one ulp always. The uncorrected a * r is not only
// less accurate but biased: rcp.approx errs to the same side over whole
// ranges of inputs (measured on GB300 over [0.5, 2), per 1/64 of the range:
// mean relative errors from -0.24 to +0.38 units of 2^-24, where a correctly
// rounded reciprocal averages 0.0002). A primitive velocity m / Sigma
// with such a bias advects every density feature at a slightly wrong speed,
// an error that grows linearly with time.
__device__ __forceinline__ float div_corrected(float a, float b, float r)
{
    const float q0 = __fmul_rn(a, r);
    return __fmaf_rn(r, __fmaf_rn(-b, q0, a), q0);
}

// Three-input minimum and maximum (PTX ISA 8.8, sm_100 and later).
__device__ __forceinline__ float min3f(float a, float b, float c)
{
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

__device__ __forceinline__ float max3f(float a, float b, float c)
{
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

__device__ inline float sqrt_fast(float x)
{
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ inline float rsqrt_fast(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ inline float exp_fast(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x * 1.4426950408889634f));
    return y;
}

} // namespace mara
