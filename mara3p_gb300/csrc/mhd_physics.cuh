// Pointwise ideal-MHD physics on the device, shared by the constrained-
// transport stage kernels (mhd.cu) and the reference's split and pointwise
// entry points (mhd_v2.cu): primitive record, fast-magnetosonic wavespeeds,
// conserved densities, HLLE flux with the transverse E-field, and the FP64
// primitive recovery, each following src/physics_mhd.hpp (cited per function).
// R = double keeps the reference's evaluation order; R = float is the mixed
// path's arithmetic (single MUFU division and square root).
#pragma once
#include <cuda_runtime.h>
#include "mixed_math.cuh"

namespace mara {
namespace mhd {

template<typename R>
struct Prim { R d, v[3], p, b[3]; };

// Division and square root: IEEE in FP64 (the reference's arithmetic), single
// MUFU approximations in the mixed path's FP32 (relative error ~1e-7).
__device__ inline double qdiv(double a, double b) { return a / b; }
__device__ inline float qdiv(float a, float b) { return a * rcp_fast(b); }
__device__ inline double qsqrt(double a) { return sqrt(a); }
__device__ inline float qsqrt(float a) { return sqrt_fast(a); }

template<typename R>
__device__ inline R sum3(const R a[3], const R b[3]) { return ((R(0) + a[0] * b[0]) + a[1] * b[1]) + a[2] * b[2]; }

__device__ inline double plm(double yl, double y0, double yr, double theta)
{
    double a = (y0 - yl) * theta, b = (yr - yl) * 0.5, c = (yr - y0) * theta;
    double m = fmin(fmin(fabs(a), fabs(b)), fabs(c));
    long long sa = __double_as_longlong(a), sb = __double_as_longlong(b), sc = __double_as_longlong(c);
    return ((sa ^ sb) | (sa ^ sc)) < 0 ? 0.0 : copysign(m, a);
}

__device__ inline float plm(float yl, float y0, float yr, float theta)
{
    float a = (y0 - yl) * theta, b = (yr - yl) * 0.5f, c = (yr - y0) * theta;
    float m = fminf(fminf(fabsf(a), fabsf(b)), fabsf(c));
    int sa = __float_as_int(a), sb = __float_as_int(b), sc = __float_as_int(c);
    return ((sa ^ sb) | (sa ^ sc)) < 0 ? 0.0f : copysignf(m, a);
}

// Twice plm(float) in one multiply: for a = y0 - yl, b = yr - yl, c = yr - y0,
// 2 minmod(theta a, b / 2, theta c) = sign x min(2 theta min(|a|, |c|), |b|).
// Scaling by two and taking minima commute with rounding, so this is exactly
// twice the three-multiply form (normal values; the signs tested are those of
// a, b, c, which scaling by theta > 0 keeps), and y +- 0.25 x plm2 rounds to
// the same float as y +- 0.5 x plm. (The median form of the minidisk sweeps,
// in three-input minima and maxima, measured 0.4% slower here.)
__device__ inline float plm2(float yl, float y0, float yr, float two_theta)
{
    const float a = y0 - yl, b = yr - yl, c = yr - y0;
    const float m = fminf(two_theta * fminf(fabsf(a), fabsf(c)), fabsf(b));
    const int sa = __float_as_int(a), sb = __float_as_int(b), sc = __float_as_int(c);
    return ((sa ^ sb) | (sa ^ sc)) < 0 ? 0.0f : copysignf(m, a);
}

// Component `axis` of v. The FP32 path takes the normal components this way
// rather than as a dot product with the unit normal: the products by 0 and 1
// change nothing but the sign of a zero, and cost six FMAs per call.
template<typename R>
__device__ __forceinline__ R pick(const R v[3], int axis) { return axis == 0 ? v[0] : (axis == 1 ? v[1] : v[2]); }

// n x v for n the unit normal along AXIS, in the FP32 path without the
// products by 0 and 1 (equal but for the sign of a zero)
template<int AXIS, typename R>
__device__ __forceinline__ void normal_cross(const R v[3], R out[3])
{
    out[AXIS] = R(0);
    out[(AXIS + 1) % 3] = -v[(AXIS + 2) % 3];
    out[(AXIS + 2) % 3] = v[(AXIS + 1) % 3];
}

// fast_speed_squared / outer_wavespeeds (physics_mhd.hpp:216-237)
template<typename R>
__device__ inline void outer_wavespeeds(const Prim<R>& p, int axis, R gm, R& am, R& ap)
{
    constexpr bool F32 = sizeof(R) == sizeof(float);
    const R n[3] = {R(axis == 0), R(axis == 1), R(axis == 2)};
    const R cs2 = qdiv(gm * p.p, p.d);
    const R va2 = qdiv(sum3(p.b, p.b), p.d);
    const R bn = F32 ? pick(p.b, axis) : sum3(p.b, n);
    const R van2 = qdiv(bn * bn, p.d);
    const R cf2 = cs2 + va2;
    R disc = cf2 * cf2 - R(4) * cs2 * van2;
    if (sizeof(R) == sizeof(float)) disc = fmax(disc, R(0));   // FP32 rounding can dip below zero
    const R cg2 = qsqrt(disc);
    const R cf = qsqrt(R(0.5) * (cf2 + cg2));
    const R vn = F32 ? pick(p.v, axis) : sum3(n, p.v);
    am = vn - cf;
    ap = vn + cf;
}

template<typename R>
__device__ inline R fastest_speed(const Prim<R>& p, R gm)
{
    R m[3], q[3];
    for (int a = 0; a < 3; ++a) outer_wavespeeds(p, a, gm, m[a], q[a]);
    return fmax(fmax(fmax(fabs(m[0]), fabs(q[0])), fmax(fabs(m[1]), fabs(q[1]))), fmax(fabs(m[2]), fabs(q[2])));
}

// conserved_density (physics_mhd.hpp:305-318)
template<typename R>
__device__ inline void conserved(const Prim<R>& p, R gm, R u[5])
{
    u[0] = p.d;
    u[1] = p.d * p.v[0];
    u[2] = p.d * p.v[1];
    u[3] = p.d * p.v[2];
    u[4] = R(0.5) * p.d * sum3(p.v, p.v) + qdiv(p.p, gm - R(1)) + R(0.5) * sum3(p.b, p.b);
}

// HLLE flux and E-field (physics_mhd.hpp:324-390), `axis` normal, bl the face B.
template<typename R, int AXIS>
__device__ inline void riemann_hlle(Prim<R> pl, Prim<R> pr, R bl, R gm, R F[5], R Et[2])
{
    pl.b[AXIS] = bl;   // with_longitudinal_field: (b - (b.n) n) + bl n
    pr.b[AXIS] = bl;
    R ul[5], ur[5], fl[5], fr[5];
    conserved(pl, gm, ul);
    conserved(pr, gm, ur);
    auto flux = [gm] (const Prim<R>& p, const R u[5], R f[5]) {
        const R bn = p.b[AXIS], vn = p.v[AXIS];
        const R pt = p.p + R(0.5) * sum3(p.b, p.b);
        const R bv = sum3(p.b, p.v);
        f[0] = vn * u[0];
        for (int k = 0; k < 3; ++k) f[1 + k] = vn * u[1 + k] + (k == AXIS ? pt : R(0)) + -bn * p.b[k];
        f[4] = vn * u[4] + pt * vn + -bn * bv;
    };
    flux(pl, ul, fl);
    flux(pr, ur, fr);
    R alm, alp, arm, arp;
    outer_wavespeeds(pl, AXIS, gm, alm, alp);
    outer_wavespeeds(pr, AXIS, gm, arm, arp);
    const R ap = fmax(R(0), fmax(alp, arp));
    const R am = fmin(R(0), fmin(alm, arm));
    for (int k = 0; k < 5; ++k) F[k] = qdiv(ap * fl[k] - am * fr[k] - (ul[k] - ur[k]) * ap * am, ap - am);
    // induction = n x E with E = -(v x B); E-field of the face = -(n x hll_induction)
    constexpr bool F32 = sizeof(R) == sizeof(float);
    auto induction = [] (const Prim<R>& p, R I[3]) {
        const R e[3] = {-(p.v[1] * p.b[2] - p.v[2] * p.b[1]), -(p.v[2] * p.b[0] - p.v[0] * p.b[2]),
                        -(p.v[0] * p.b[1] - p.v[1] * p.b[0])};
        const R n[3] = {R(AXIS == 0), R(AXIS == 1), R(AXIS == 2)};
        if (F32)
        {
            normal_cross<AXIS>(e, I);
            return;
        }
        I[0] = n[1] * e[2] - n[2] * e[1];
        I[1] = n[2] * e[0] - n[0] * e[2];
        I[2] = n[0] * e[1] - n[1] * e[0];
    };
    R il[3], ir[3], hi[3];
    induction(pl, il);
    induction(pr, ir);
    for (int k = 0; k < 3; ++k) hi[k] = qdiv(ap * il[k] - am * ir[k] - (pl.b[k] - pr.b[k]) * ap * am, ap - am);
    const R n[3] = {R(AXIS == 0), R(AXIS == 1), R(AXIS == 2)};
    R c[3] = {n[1] * hi[2] - n[2] * hi[1], n[2] * hi[0] - n[0] * hi[2], n[0] * hi[1] - n[1] * hi[0]};
    if (F32) normal_cross<AXIS>(hi, c);
    // transverse components in increasing axis order
    Et[0] = -c[AXIS == 0 ? 1 : 0];
    Et[1] = -c[AXIS == 2 ? 1 : 2];
}

// recover_primitive (physics_mhd.hpp:290-303) in FP64 from the conserved
// densities u = (D, S1, S2, S3, E) and the cell-centred field b; false where
// the reference throws (negative density or pressure). The arithmetic order
// is the stage kernels' (kinetic energy as |S|^2 / (2 D)).
__device__ inline bool recover_primitive(const double u[5], const double b[3], double gamma, Prim<double>& p)
{
    const double d = u[0];
    const double S[3] = {u[1], u[2], u[3]};
    const double kin = 0.5 * sum3(S, S) / d;
    const double mag = 0.5 * sum3(b, b);
    const double pg = (u[4] - kin - mag) * (gamma - 1);
    p.d = d;
    for (int q = 0; q < 3; ++q)
    {
        p.v[q] = S[q] / d;
        p.b[q] = b[q];
    }
    p.p = pg;
    return !(d < 0.0 || pg < 0.0);
}

} // namespace mhd
} // namespace mara
