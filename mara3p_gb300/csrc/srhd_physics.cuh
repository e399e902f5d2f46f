// SRHD device physics shared by the batch recovery (srhd.cu) and the 2D
// scheme (srhd_tube.cu), c = 1, in the reference's evaluation order
// (src/physics_srhd.hpp): recover_primitive :231-285, conserved_density
// :291-304, flux :310-324, outer_wavespeeds :182-195, HLLE :377-420.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "mixed_math.cuh"

namespace mara {
namespace srhd {

struct Zone { double D, S1, S2, S3, tau; };

// Newton on p from p_start (physics_srhd.hpp:231-285), in resumable pieces:
// newton_steps runs the reference's iterations from (p, iteration) while
// iteration <= iter_max and iteration < stop, returning true (with W0) once
// the stopping rule holds (|f| < 1e-12, or 1e-8 on the last allowed
// iteration); resuming from the same (p, iteration) gives the same iterates
// as one uninterrupted run. newton_finish applies the floor and forms the
// primitives. newton is the whole recovery: status 0 ok / 1 not converged /
// 2 non-positive pressure; it writes the primitive (rho, u1, u2, u3, p) and
// the number of iterations run.
__device__ inline bool newton_steps(const Zone& z, double gm, double& p, int& iteration, int iter_max, int stop,
                                    double& W0)
{
    const double c2 = 1.0;
    const double tol = 1e-12;
    const double D = z.D, tau = z.tau;
    const double SS = __dadd_rn(__dadd_rn(__dadd_rn(0.0, __dmul_rn(z.S1, z.S1)), __dmul_rn(z.S2, z.S2)),
                                __dmul_rn(z.S3, z.S3));
    const double Dc2 = D;   // D * c^2
    const double gm1 = __dadd_rn(gm, -1.0);
    const double b2max = 1.0 - 1e-10;
    while (iteration <= iter_max && iteration < stop)
    {
        double Et = __dadd_rn(__dadd_rn(tau, p), Dc2);
        double b2 = fmin(__ddiv_rn(__ddiv_rn(SS, Et), Et), b2max);
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
            return true;
        }
        ++iteration;
    }
    return false;
}

__device__ inline int newton_finish(const Zone& z, double temperature_floor, double p, double W0, bool found,
                                    int iteration, double prim[5], int& iterations)
{
    const double D = z.D, tau = z.tau;
    const double Dc2 = D;
    iterations = found ? iteration + 1 : iteration;
    if (temperature_floor > 0.0)
        p = fmax(p, __dmul_rn(temperature_floor, D));
    if (!found) return 1;
    if (temperature_floor <= 0.0 && p <= 0.0) return 2;
    double Et = __dadd_rn(__dadd_rn(tau, Dc2), p);
    prim[0] = __ddiv_rn(D, W0);
    prim[1] = __ddiv_rn(__dmul_rn(W0, z.S1), Et);   // the reference's trailing * c is a * 1
    prim[2] = __ddiv_rn(__dmul_rn(W0, z.S2), Et);
    prim[3] = __ddiv_rn(__dmul_rn(W0, z.S3), Et);
    prim[4] = p;
    return 0;
}

__device__ inline int newton(const Zone& z, double gm, double temperature_floor, double p_start, int iter_max,
                             double prim[5], int& iterations)
{
    int iteration = 0;
    double W0 = 1.0, p = p_start;
    const bool found = newton_steps(z, gm, p, iteration, iter_max, iter_max + 1, W0);
    return newton_finish(z, temperature_floor, p, W0, found, iteration, prim, iterations);
}

// FP64 reciprocal and inverse square root for the seeded polish: an FP32
// seed (relative error ~2^-22) and two Newton-Raphson steps, each of which
// squares the relative error (y <- y + y (1 - b y); y <- y (3/2 - x y^2 / 2)),
// so the result is within a few ulp of the exact value. Arguments must lie in
// the FP32 normal range, as the polish's quantities do; anything else gives
// NaN or infinity and the zone falls back to the exact iteration.
__device__ inline double rcp_nr(double b)
{
    double y = f2d(rcp_fast(d2f(b)));
    y = fma(y, fma(-b, y, 1.0), y);
    y = fma(y, fma(-b, y, 1.0), y);
    return y;
}

__device__ inline double rsqrt_nr(double x)
{
    const double h = 0.5 * x;
    double y = f2d(rsqrt_fast(d2f(x)));
    y = y * fma(-h * y, y, 1.5);
    y = y * fma(-h * y, y, 1.5);
    return y;
}

// The Newton iteration of newton() from a seeded pressure with the same
// stopping rule (|f| < 1e-12, 1e-8 on the last allowed iteration) and the
// same final primitives, its update rearranged to three reciprocals and one
// inverse square root per iteration instead of eight divisions and a square
// root. The seeded paths use it; the reference's own start (newton) keeps the
// reference's arithmetic bit for bit.
// newton_fast in resumable pieces. newton_fast_steps runs the iterations
// from (p, iteration) while iteration <= iter_max and iteration < stop,
// returning true (with W0) once the stopping rule holds; a caller may stop
// early and resume later from the same (p, iteration), which gives the same
// iterates as one uninterrupted run. newton_fast_finish applies the floor and
// forms the primitives.
__device__ inline bool newton_fast_steps(const Zone& z, double gm, double& p, int& iteration, int iter_max, int stop,
                                         double& W0)
{
    const double tol = 1e-12;
    const double D = z.D, tau = z.tau;
    const double SS = z.S1 * z.S1 + z.S2 * z.S2 + z.S3 * z.S3;
    const double iD = rcp_nr(D);
    const double gm1 = gm - 1.0;
    const double b2max = 1.0 - 1e-10;
    while (iteration <= iter_max && iteration < stop)
    {
        const double Et = (tau + p) + D;
        const double iE = rcp_nr(Et);
        const double b2 = fmin(SS * iE * iE, b2max);
        const double ib = 1.0 - b2;
        const double W = rsqrt_nr(ib);                 // 1 / sqrt(1 - b2)
        const double W2 = W * W;
        const double iW = ib * W;                      // sqrt(1 - b2)
        const double e = ((tau + D * (1.0 - W)) + p * (1.0 - W2)) * iW * iD;
        const double d = D * iW;
        const double pWD = p * W * iD;                 // p / d
        const double h = (1.0 + e) + pWD;
        const double a2 = gm * pWD * rcp_nr(h);        // gm p / (d h)
        const double f = d * e * gm1 - p;
        const double g = b2 * a2 - 1.0;
        p = fma(-f, rcp_nr(g), p);
        if (fabs(f) < tol || (fabs(f) < tol * 1e4 && iteration == iter_max))
        {
            W0 = W;
            return true;
        }
        ++iteration;
    }
    return false;
}

__device__ inline int newton_fast_finish(const Zone& z, double temperature_floor, double p, double W0, bool found,
                                         int iteration, double prim[5], int& iterations)
{
    const double D = z.D, tau = z.tau;
    iterations = found ? iteration + 1 : iteration;
    if (temperature_floor > 0.0) p = fmax(p, temperature_floor * D);
    if (!found) return 1;
    if (temperature_floor <= 0.0 && p <= 0.0) return 2;
    const double Et = __dadd_rn(__dadd_rn(tau, D), p);
    prim[0] = __ddiv_rn(D, W0);
    prim[1] = __ddiv_rn(__dmul_rn(W0, z.S1), Et);
    prim[2] = __ddiv_rn(__dmul_rn(W0, z.S2), Et);
    prim[3] = __ddiv_rn(__dmul_rn(W0, z.S3), Et);
    prim[4] = p;
    return 0;
}

__device__ inline int newton_fast(const Zone& z, double gm, double temperature_floor, double p_start, int iter_max,
                                  double prim[5], int& iterations)
{
    int iteration = 0;
    double W0 = 1.0, p = p_start;
    const bool found = newton_fast_steps(z, gm, p, iteration, iter_max, iter_max + 1, W0);
    return newton_fast_finish(z, temperature_floor, p, W0, found, iteration, prim, iterations);
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

// Explicitly rounded arithmetic, no contraction: in FP64 the fluxes below
// equal the reference's (compiled without FMA contraction) bit for bit; in
// FP32 they are the mixed path's. The reference's factors and divisors of
// c = 1 (x * 1, x / 1, 1 * 1) are exact identities and are left out.
__device__ inline double rmul(double a, double b) { return __dmul_rn(a, b); }
__device__ inline double radd(double a, double b) { return __dadd_rn(a, b); }
__device__ inline double rsub(double a, double b) { return __dsub_rn(a, b); }
__device__ inline double rdiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ inline double rsqrt_rn(double a) { return __dsqrt_rn(a); }
__device__ inline float rmul(float a, float b) { return __fmul_rn(a, b); }
__device__ inline float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ inline float rsub(float a, float b) { return __fsub_rn(a, b); }
__device__ inline float rdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ inline float rsqrt_rn(float a) { return __fsqrt_rn(a); }

// 0 + u1^2 + u2^2 + u3^2 (physics_srhd.hpp gamma_beta_squared)
template<typename R>
__device__ inline R gamma_beta_squared(const SPrim<R>& p)
{
    return radd(radd(radd(R(0), rmul(p.u[0], p.u[0])), rmul(p.u[1], p.u[1])), rmul(p.u[2], p.u[2]));
}

template<typename R>
__device__ inline R lorentz_factor(const SPrim<R>& p) { return rsqrt_rn(radd(R(1), gamma_beta_squared(p))); }

// rho c^2 + p (1 + 1/(gamma - 1))
template<typename R>
__device__ inline R enthalpy_density(const SPrim<R>& p, R gm)
{
    return radd(p.rho, rmul(p.p, radd(R(1), rdiv(R(1), rsub(gm, R(1))))));
}

// conserved_density (physics_srhd.hpp:291-304)
template<typename R>
__device__ inline void cons_of(const SPrim<R>& p, R gm, R u[5])
{
    const R W = lorentz_factor(p);
    const R D = rmul(p.rho, W);
    const R h = rdiv(enthalpy_density(p, gm), p.rho);
    u[0] = D;
    for (int k = 0; k < 3; ++k) u[1 + k] = rmul(rmul(D, h), p.u[k]);
    u[4] = rsub(rmul(D, rsub(rmul(h, W), R(1))), p.p);
}

// normal three-velocity 0 + n.v along axis (0, 1, 2); the terms of the other
// two axes are exact zeros for finite velocities and are left out
template<typename R>
__device__ inline R normal_velocity(const SPrim<R>& p, int axis)
{
    return radd(R(0), rdiv(p.u[axis], lorentz_factor(p)));
}

// flux (physics_srhd.hpp:310-324)
template<typename R>
__device__ inline void flux_of(const SPrim<R>& p, const R u[5], int axis, R f[5])
{
    const R vn = normal_velocity(p, axis);
    const R pt[5] = {R(0), rmul(p.p, R(axis == 0)), rmul(p.p, R(axis == 1)), rmul(p.p, R(axis == 2)),
                     rmul(p.p, vn)};
    for (int k = 0; k < 5; ++k) f[k] = radd(rmul(vn, u[k]), pt[k]);
}

// outer_wavespeeds (physics_srhd.hpp:182-195)
template<typename R>
__device__ inline void outer_speeds(const SPrim<R>& p, int axis, R gm, R& am, R& ap)
{
    const R a2 = rdiv(rmul(gm, p.p), enthalpy_density(p, gm));
    const R uu = gamma_beta_squared(p);
    const R vn = normal_velocity(p, axis);
    const R bn = vn;
    const R bb = rdiv(uu, radd(R(1), uu));
    const R b2 = rmul(bn, bn);
    R disc = rmul(rmul(a2, rsub(R(1), bb)), rsub(rsub(R(1), rmul(bb, a2)), rmul(b2, rsub(R(1), a2))));
    if (sizeof(R) == sizeof(float)) disc = fmax(disc, R(0));   // FP32 rounding can dip below zero
    const R k0 = rsqrt_rn(disc);
    const R den = rsub(R(1), rmul(bb, a2));
    const R vna = rmul(vn, rsub(R(1), a2));
    am = rdiv(rsub(vna, k0), den);
    ap = rdiv(radd(vna, k0), den);
}

// (ar fl - al fr - (ul - ur) ar al) / (ar - al)
template<typename R>
__device__ inline R hll_average(R fl, R fr, R ul, R ur, R al, R ar)
{
    return rdiv(rsub(rsub(rmul(ar, fl), rmul(al, fr)), rmul(rmul(rsub(ul, ur), ar), al)), rsub(ar, al));
}

// riemann_hlle (fixed face, physics_srhd.hpp:395-400, 489-497) along axis
template<typename R>
__device__ inline void hlle(const SPrim<R>& pl, const SPrim<R>& pr, int axis, R gm, R F[5])
{
    R ul[5], ur[5], fl[5], fr[5];
    cons_of(pl, gm, ul);
    cons_of(pr, gm, ur);
    flux_of(pl, ul, axis, fl);
    flux_of(pr, ur, axis, fr);
    R alm, alp, arm, arp;
    outer_speeds(pl, axis, gm, alm, alp);
    outer_speeds(pr, axis, gm, arm, arp);
    const R ar = fmax(alp, arp);
    const R al = fmin(alm, arm);
    if (R(0) < al) { for (int k = 0; k < 5; ++k) F[k] = fl[k]; return; }
    if (R(0) > ar) { for (int k = 0; k < 5; ++k) F[k] = fr[k]; return; }
    for (int k = 0; k < 5; ++k) F[k] = hll_average(fl[k], fr[k], ul[k], ur[k], al, ar);
}

// riemann_hllc (fixed face, physics_srhd.hpp:401-487; Mignone & Bodo 2005)
// along axis. Returns 1 where the reference throws (contact speed NaN or
// beyond 1e3); F then holds the HLLE flux.
template<typename R>
__device__ inline int hllc(const SPrim<R>& pl, const SPrim<R>& pr, int axis, R gm, R F[5])
{
    R ul[5], ur[5], fl[5], fr[5];
    cons_of(pl, gm, ul);
    cons_of(pr, gm, ur);
    flux_of(pl, ul, axis, fl);
    flux_of(pr, ur, axis, fr);
    R alm, alp, arm, arp;
    outer_speeds(pl, axis, gm, alm, alp);
    outer_speeds(pr, axis, gm, arm, arp);
    const R ar = fmax(alp, arp);
    const R al = fmin(alm, arm);
    R u_hll[5], f_hll[5];
    for (int k = 0; k < 5; ++k)
    {
        u_hll[k] = rdiv(radd(rsub(rmul(ar, ur[k]), rmul(al, ul[k])), rsub(fl[k], fr[k])), rsub(ar, al));
        f_hll[k] = hll_average(fl[k], fr[k], ul[k], ur[k], al, ar);
    }
    const R n[3] = {R(axis == 0), R(axis == 1), R(axis == 2)};
    const R ue_hll = radd(u_hll[4], u_hll[0]);
    const R fe_hll = radd(f_hll[4], f_hll[0]);
    const R um_hll = radd(radd(radd(R(0), rmul(u_hll[1], n[0])), rmul(u_hll[2], n[1])), rmul(u_hll[3], n[2]));
    const R fm_hll = radd(radd(radd(R(0), rmul(f_hll[1], n[0])), rmul(f_hll[2], n[1])), rmul(f_hll[3], n[2]));
    const R a = fe_hll;
    const R b = rsub(-fm_hll, ue_hll);
    const R c = um_hll;
    const R d = rsub(rmul(b, b), rmul(rmul(R(4), a), c));
    const R as = d < R(0) ? R(0)
               : (fabs(a) > R(1e-8) ? rdiv(rsub(-b, rsqrt_rn(d)), rmul(R(2), a)) : rdiv(-c, b));
    if (isnan(as) || as < R(-1e3) || as > R(1e3))
    {
        for (int k = 0; k < 5; ++k) F[k] = f_hll[k];
        if (R(0) < al) for (int k = 0; k < 5; ++k) F[k] = fl[k];
        if (R(0) > ar) for (int k = 0; k < 5; ++k) F[k] = fr[k];
        return 1;
    }
    const R ps = radd(rmul(-fe_hll, as), fm_hll);
    auto star = [&](const R u[5], const R f[5], const SPrim<R>& p, R s) {
        const R v = normal_velocity(p, axis);
        const R e = radd(u[4], u[0]);
        const R m = radd(radd(radd(R(0), rmul(u[1], n[0])), rmul(u[2], n[1])), rmul(u[3], n[2]));
        const R sv = rsub(s, v), sa = rsub(s, as);
        const R es = rdiv(rsub(radd(rmul(e, sv), rmul(ps, as)), rmul(p.p, v)), sa);
        const R ms = rdiv(rsub(radd(rmul(m, sv), ps), p.p), sa);
        const R Ds = rdiv(rmul(u[0], sv), sa);
        R us[5];
        us[0] = Ds;
        for (int k = 0; k < 3; ++k)
        {
            const R nk = rsub(u[1 + k], rmul(m, n[k]));
            const R ns = rdiv(rmul(nk, sv), sa);
            us[1 + k] = radd(rmul(ms, n[k]), ns);
        }
        us[4] = rsub(es, Ds);
        for (int k = 0; k < 5; ++k) F[k] = rsub(radd(f[k], rmul(s, rsub(us[k], u[k]))), rmul(R(0), us[k]));
    };
    if (R(0) <= al) { for (int k = 0; k < 5; ++k) F[k] = fl[k]; return 0; }
    if (R(0) >= ar) { for (int k = 0; k < 5; ++k) F[k] = fr[k]; return 0; }
    if (R(0) <= as) star(ul, fl, pl, al);
    else star(ur, fr, pr, ar);
    return 0;
}

} // namespace srhd
} // namespace mara
