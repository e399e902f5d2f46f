// SRHD device physics shared by the batch recovery (srhd.cu) and the 2D
// scheme (srhd_tube.cu), c = 1, in the reference's evaluation order
// (src/physics_srhd.hpp): recover_primitive :231-285, conserved_density
// :291-304, flux :310-324, outer_wavespeeds :182-195, HLLE :377-420.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace mara {
namespace srhd {

struct Zone { double D, S1, S2, S3, tau; };

// Newton on p from p_start (physics_srhd.hpp:231-285). Returns status
// 0 ok / 1 not converged / 2 non-positive pressure; writes the primitive
// (rho, u1, u2, u3, p) and the number of iterations run.
__device__ inline int newton(const Zone& z, double gm, double temperature_floor, double p_start, int iter_max,
                             double prim[5], int& iterations)
{
    const double c2 = 1.0;
    const double tol = 1e-12;
    const double D = z.D, tau = z.tau;
    const double SS = __dadd_rn(__dadd_rn(__dadd_rn(0.0, __dmul_rn(z.S1, z.S1)), __dmul_rn(z.S2, z.S2)),
                                __dmul_rn(z.S3, z.S3));
    const double Dc2 = __dmul_rn(D, c2);
    const double gm1 = __dadd_rn(gm, -1.0);
    const double b2max = 1.0 - 1e-10;
    bool found = false;
    int iteration = 0;
    double W0 = 1.0;
    double p = p_start;

    while (iteration <= iter_max)
    {
        double Et = __dadd_rn(__dadd_rn(tau, p), Dc2);
        double b2 = fmin(__ddiv_rn(__ddiv_rn(__dmul_rn(SS, c2), Et), Et), b2max);
        double W2 = __ddiv_rn(1.0, __dadd_rn(1.0, -b2));
        double W = __dsqrt_rn(W2);
        double e = __ddiv_rn(__dadd_rn(__dadd_rn(tau, __dmul_rn(Dc2, __dadd_rn(1.0, -W))), __dmul_rn(p, __dadd_rn(1.0, -W2))),
                             __dmul_rn(D, W));
        double d = __ddiv_rn(D, W);
        double h = __dadd_rn(__dadd_rn(c2, e), __ddiv_rn(p, d));
        double a2 = __ddiv_rn(__dmul_rn(gm, p), __dmul_rn(d, h));
        double f = __dadd_rn(__dmul_rn(__dmul_rn(d, e), gm1), -p);
        double g = __dadd_rn(__dmul_rn(b2, a2), -1.0);

        p = __dadd_rn(p, -__ddiv_rn(f, g));

        if (fabs(f) < tol || (fabs(f) < tol * 1e4 && iteration == iter_max))
        {
            W0 = W;
            found = true;
            break;
        }
        ++iteration;
    }
    iterations = found ? iteration + 1 : iteration;
    if (temperature_floor > 0.0)
        p = fmax(p, __dmul_rn(__dmul_rn(temperature_floor, D), c2));
    if (!found) return 1;
    if (temperature_floor <= 0.0 && p <= 0.0) return 2;
    double Et = __dadd_rn(__dadd_rn(tau, Dc2), p);
    prim[0] = __ddiv_rn(D, W0);
    prim[1] = __dmul_rn(__ddiv_rn(__dmul_rn(W0, z.S1), Et), 1.0);
    prim[2] = __dmul_rn(__ddiv_rn(__dmul_rn(W0, z.S2), Et), 1.0);
    prim[3] = __dmul_rn(__ddiv_rn(__dmul_rn(W0, z.S3), Et), 1.0);
    prim[4] = p;
    return 0;
}

// The same Newton update in FP32, used to sharpen a pressure guess cheaply
// before the FP64 polish. Returns the guess unchanged if it goes bad.
__device__ inline double refine_fp32(const Zone& z, double gm, double p0, int iters)
{
    const float D = float(z.D), tau = float(z.tau), g = float(gm);
    const float SS = float(z.S1) * float(z.S1) + float(z.S2) * float(z.S2) + float(z.S3) * float(z.S3);
    float p = float(p0);
    for (int k = 0; k < iters; ++k)
    {
        float Et = tau + p + D;
        float b2 = fminf(SS / (Et * Et), 1.0f - 1e-7f);
        float W2 = 1.0f / (1.0f - b2);
        float W = sqrtf(W2);
        float e = (tau + D * (1.0f - W) + p * (1.0f - W2)) / (D * W);
        float d = D / W;
        float h = 1.0f + e + p / d;
        float a2 = g * p / (d * h);
        float f = d * e * (g - 1.0f) - p;
        float gg = b2 * a2 - 1.0f;
        float pn = p - f / gg;
        if (!(pn > 0.0f) || !isfinite(pn)) break;
        p = pn;
    }
    return double(p);
}

// srhd::conserved_density (src/physics_srhd.hpp:291-304), c = 1
__device__ inline void conserved_density(const double p[5], double gm, double u[5])
{
    const double W = sqrt(1.0 + (p[1] * p[1] + p[2] * p[2] + p[3] * p[3]));
    const double D = p[0] * W;
    const double h = (p[0] * 1.0 + p[4] * (1.0 + 1.0 / (gm - 1.0))) / p[0];
    u[0] = D;
    u[1] = D * h * p[1] / 1.0;
    u[2] = D * h * p[2] / 1.0;
    u[3] = D * h * p[3] / 1.0;
    u[4] = D * (h * W - 1.0 * 1.0) - p[4];
}

template<typename R>
struct SPrim { R rho, u[3], p; };

template<typename R>
__device__ inline R gamma_beta_squared(const SPrim<R>& p) { return p.u[0] * p.u[0] + p.u[1] * p.u[1] + p.u[2] * p.u[2]; }

template<typename R>
__device__ inline void cons_of(const SPrim<R>& p, R gm, R u[5])
{
    const R W = sqrt(R(1) + gamma_beta_squared(p));
    const R D = p.rho * W;
    const R h = (p.rho * R(1) + p.p * (R(1) + R(1) / (gm - R(1)))) / p.rho;
    u[0] = D;
    for (int k = 0; k < 3; ++k) u[1 + k] = D * h * p.u[k] / R(1);
    u[4] = D * (h * W - R(1) * R(1)) - p.p;
}

// normal three-velocity along axis (0, 1, 2)
template<typename R>
__device__ inline R normal_velocity(const SPrim<R>& p, int axis)
{
    const R W = sqrt(R(1) + gamma_beta_squared(p));
    return R(1) * p.u[axis] / W;
}

template<typename R>
__device__ inline void outer_speeds(const SPrim<R>& p, int axis, R gm, R& am, R& ap)
{
    const R H = p.rho * R(1) + p.p * (R(1) + R(1) / (gm - R(1)));
    const R a2 = gm * R(1) * p.p / H / R(1);
    const R uu = gamma_beta_squared(p);
    const R vn = normal_velocity(p, axis);
    const R bn = vn / R(1);
    const R bb = uu / (R(1) + uu);
    const R b2 = bn * bn;
    R disc = a2 * (R(1) - bb) * (R(1) - bb * a2 - b2 * (R(1) - a2));
    if (sizeof(R) == sizeof(float)) disc = fmax(disc, R(0));   // FP32 rounding can dip below zero
    const R k0 = sqrt(disc) * R(1);
    am = (vn * (R(1) - a2) - k0) / (R(1) - bb * a2);
    ap = (vn * (R(1) - a2) + k0) / (R(1) - bb * a2);
}

// riemann_hlle (fixed face, physics_srhd.hpp:395-400, 489-497) along axis
template<typename R>
__device__ inline void hlle(const SPrim<R>& pl, const SPrim<R>& pr, int axis, R gm, R F[5])
{
    R ul[5], ur[5], fl[5], fr[5];
    cons_of(pl, gm, ul);
    cons_of(pr, gm, ur);
    const R vl = normal_velocity(pl, axis), vr = normal_velocity(pr, axis);
    for (int k = 0; k < 5; ++k)
    {
        const R ptl = k == 0 ? R(0) * R(0) : (k == 4 ? pl.p * vl : (k - 1 == axis ? pl.p : R(0)));
        const R ptr = k == 0 ? R(0) * R(0) : (k == 4 ? pr.p * vr : (k - 1 == axis ? pr.p : R(0)));
        fl[k] = vl * ul[k] + ptl;
        fr[k] = vr * ur[k] + ptr;
    }
    R alm, alp, arm, arp;
    outer_speeds(pl, axis, gm, alm, alp);
    outer_speeds(pr, axis, gm, arm, arp);
    const R ar = fmax(alp, arp);
    const R al = fmin(alm, arm);
    if (R(0) < al) { for (int k = 0; k < 5; ++k) F[k] = fl[k]; return; }
    if (R(0) > ar) { for (int k = 0; k < 5; ++k) F[k] = fr[k]; return; }
    for (int k = 0; k < 5; ++k) F[k] = (ar * fl[k] - al * fr[k] - (ul[k] - ur[k]) * ar * al) / (ar - al);
}

} // namespace srhd
} // namespace mara
