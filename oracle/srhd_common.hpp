// ORACLE — test infrastructure only (see oracle_common.hpp).
//
// The reference's special-relativistic physics (src/physics_srhd.hpp), c = 1,
// restated for the SRHD oracles (srhd_oracle.cpp, sedov_oracle.cpp):
//   recover_primitive     :231-285  Newton on p, 50+1 iterations, |f| < 1e-12
//                                   (1e-8 on the last iteration)
//   conserved_density     :291-304
//   flux                  :310-324
//   outer_wavespeeds      :182-195
//   riemann_solver        :377-487  (HLLE and the HLLC modes, Mignone & Bodo 2005)
// Arithmetic keeps the reference's evaluation order.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>

namespace oracle {
namespace srhd {

struct Prim { double rho, u1, u2, u3, p; };
struct Cons { double c[5]; };

inline double gamma_beta_squared(const Prim& p) { return 0.0 + p.u1 * p.u1 + p.u2 * p.u2 + p.u3 * p.u3; }
inline double lorentz_factor(const Prim& p) { return std::sqrt(1.0 + gamma_beta_squared(p)); }
inline double enthalpy_density(const Prim& p, double gm) { return p.rho * 1.0 + p.p * (1.0 + 1.0 / (gm - 1.0)); }

inline double normal_velocity(const Prim& p, int axis)
{
    double W = lorentz_factor(p);
    double v1 = 1.0 * p.u1 / W, v2 = 1.0 * p.u2 / W, v3 = 1.0 * p.u3 / W;
    double n1 = axis == 1, n2 = axis == 2, n3 = axis == 3;
    return 0.0 + n1 * v1 + n2 * v2 + n3 * v3;
}

inline Cons conserved_density(const Prim& p, double gm)
{
    double W = lorentz_factor(p);
    double D = p.rho * W;
    double h = enthalpy_density(p, gm) / p.rho;
    return Cons{{D, D * h * p.u1 / 1.0, D * h * p.u2 / 1.0, D * h * p.u3 / 1.0, D * (h * W - 1.0 * 1.0) - p.p}};
}

inline Cons flux(const Prim& p, int axis, double gm)
{
    double vn = normal_velocity(p, axis);
    Cons u = conserved_density(p, gm);
    double n1 = axis == 1, n2 = axis == 2, n3 = axis == 3;
    double pt[5] = {0.0 * 0.0, p.p * n1, p.p * n2, p.p * n3, p.p * vn};
    Cons f;
    for (int k = 0; k < 5; ++k) f.c[k] = vn * u.c[k] + pt[k];
    return f;
}

inline void outer_wavespeeds(const Prim& p, int axis, double gm, double& am, double& ap)
{
    double a2 = gm * 1.0 * p.p / enthalpy_density(p, gm) / 1.0;
    double uu = gamma_beta_squared(p);
    double vn = normal_velocity(p, axis);
    double bn = vn / 1.0;
    double bb = uu / (1 + uu);
    double b2 = bn * bn;
    double k0 = std::sqrt(a2 * (1 - bb) * (1 - bb * a2 - b2 * (1 - a2))) * 1.0;
    am = (vn * (1 - a2) - k0) / (1 - bb * a2);
    ap = (vn * (1 - a2) + k0) / (1 - bb * a2);
}

// Returns 0 ok, 1 not converged, 2 non-positive pressure (the reference throws
// in both failure cases).
inline int recover_primitive(const double* u, double gm, double temperature_floor, double p_start,
                      Prim& out, int& iterations)
{
    const int newton_iter_max = 50;
    const double error_tolerance = 1e-12;
    const double c2 = 1.0 * 1.0;
    const double D = u[0], S1 = u[1], S2 = u[2], S3 = u[3], tau = u[4];
    const double SS = 0.0 + S1 * S1 + S2 * S2 + S3 * S3;
    bool found = false;
    int iteration = 0;
    double W0 = 1.0;
    double p = p_start;

    while (iteration <= newton_iter_max)
    {
        double Et = tau + p + D * c2;
        double b2 = std::min(SS * c2 / Et / Et, 1.0 - 1e-10);
        double W2 = 1.0 / (1.0 - b2);
        double W  = std::sqrt(W2);
        double e  = (tau + D * c2 * (1.0 - W) + p * (1.0 - W2)) / (D * W);
        double d  = D / W;
        double h  = c2 + e + p / d;
        double a2 = gm * p / (d * h);
        double f  = d * e * (gm - 1.0) - p;
        double g  = b2 * a2 - 1.0;

        p -= f / g;

        if (std::fabs(f) < error_tolerance || (std::fabs(f) < error_tolerance * 1e4 && iteration == newton_iter_max))
        {
            W0 = W;
            found = true;
            break;
        }
        ++iteration;
    }
    iterations = found ? iteration + 1 : iteration;

    if (temperature_floor > 0.0)
        p = std::max(p, temperature_floor * D * c2);
    if (!found)
        return 1;
    if (temperature_floor <= 0.0 && p <= 0.0)
        return 2;

    out.rho = D / W0;
    out.u1 = W0 * S1 / (tau + D * c2 + p) * 1.0;
    out.u2 = W0 * S2 / (tau + D * c2 + p) * 1.0;
    out.u3 = W0 * S3 / (tau + D * c2 + p) * 1.0;
    out.p = p;
    return 0;
}

inline Prim load_prim(const double* a) { return Prim{a[0], a[1], a[2], a[3], a[4]}; }

// The HLLC modes of riemann_solver (physics_srhd.hpp:351-356): fixed face,
// moving face (face_speed), and the flux across the contact with the contact
// speed (riemann_solver_mode_hllc_fluxes_across_contact_t).
enum { HLLC_FIXED = 0, HLLC_MOVING_FACE = 1, HLLC_ACROSS_CONTACT = 2 };

// riemann_solver (physics_srhd.hpp:377-487) in the fixed-face HLLE / HLLC
// modes, or (mode != HLLC_FIXED) the other HLLC modes; contact receives the
// contact speed of HLLC_ACROSS_CONTACT. Returns 1 where the reference throws
// (NaN contact speed or beyond 1e3).
inline int riemann(const Prim& pl, const Prim& pr, int axis, double gm, bool hllc, Cons& out,
                   int mode = HLLC_FIXED, double face_speed = 0.0, double* contact = nullptr)
{
    Cons ul = conserved_density(pl, gm), ur = conserved_density(pr, gm);
    Cons fl = flux(pl, axis, gm), fr = flux(pr, axis, gm);
    double alm, alp, arm, arp;
    outer_wavespeeds(pl, axis, gm, alm, alp);
    outer_wavespeeds(pr, axis, gm, arm, arp);
    double ar = std::max(alp, arp);
    double al = std::min(alm, arm);

    if (!hllc)
    {
        if (0.0 < al) { out = fl; return 0; }
        if (0.0 > ar) { out = fr; return 0; }
        for (int k = 0; k < 5; ++k)
            out.c[k] = (ar * fl.c[k] - al * fr.c[k] - (ul.c[k] - ur.c[k]) * ar * al) / (ar - al);
        return 0;
    }
    Cons u_hll, f_hll;
    for (int k = 0; k < 5; ++k)
    {
        u_hll.c[k] = (ar * ur.c[k] - al * ul.c[k] + (fl.c[k] - fr.c[k])) / (ar - al);
        f_hll.c[k] = (ar * fl.c[k] - al * fr.c[k] - (ul.c[k] - ur.c[k]) * ar * al) / (ar - al);
    }
    const double c2 = 1.0 * 1.0;
    const double n[3] = {double(axis == 1), double(axis == 2), double(axis == 3)};
    double ue_hll = u_hll.c[4] + u_hll.c[0] * c2;
    double fe_hll = f_hll.c[4] + f_hll.c[0] * c2;
    double um_hll = 0.0 + u_hll.c[1] * n[0] + u_hll.c[2] * n[1] + u_hll.c[3] * n[2];
    double fm_hll = 0.0 + f_hll.c[1] * n[0] + f_hll.c[2] * n[1] + f_hll.c[3] * n[2];
    double a = +fe_hll;
    double b = -fm_hll - ue_hll;
    double c = +um_hll;
    double d = b * b - 4.0 * a * c;
    double as = d < 0.0 ? 0.0 : (std::abs(a) > 1e-8 ? (-b - std::sqrt(d)) / (2.0 * a) : -c / b) * c2;
    if (std::isnan(as) || as < -1e3 || as > 1e3)
        return 1;
    double ps = -fe_hll * as / c2 + fm_hll;

    auto star = [&] (const Cons& u, const Cons& f, const Prim& p, double s, double w) {
        double S[3] = {u.c[1], u.c[2], u.c[3]};
        double v = normal_velocity(p, axis);
        double e = u.c[4] + u.c[0] * c2;
        double m = 0.0 + S[0] * n[0] + S[1] * n[1] + S[2] * n[2];
        double es = (e * (s - v) + ps * as - p.p * v) / (s - as);
        double ms = (m * (s - v) + ps - p.p) / (s - as);
        double Ds = u.c[0] * (s - v) / (s - as);
        Cons us;
        us.c[0] = Ds;
        for (int k = 0; k < 3; ++k)
        {
            double nk = S[k] - m * n[k];
            double ns = nk * (s - v) / (s - as);
            us.c[1 + k] = ms * n[k] + ns;
        }
        us.c[4] = es - Ds * c2;
        Cons fs;
        for (int k = 0; k < 5; ++k) fs.c[k] = (f.c[k] + s * (us.c[k] - u.c[k])) - w * us.c[k];
        return fs;
    };
    if (mode == HLLC_ACROSS_CONTACT)
    {
        out = star(ul, fl, pl, al, as);
        if (contact) *contact = as;
        return 0;
    }
    if (mode == HLLC_MOVING_FACE)
    {
        const double w = face_speed;
        if (w <= al) { for (int k = 0; k < 5; ++k) out.c[k] = fl.c[k] - w * ul.c[k]; return 0; }
        if (w >= ar) { for (int k = 0; k < 5; ++k) out.c[k] = fr.c[k] - w * ur.c[k]; return 0; }
        if (w <= as) { out = star(ul, fl, pl, al, w); return 0; }
        out = star(ur, fr, pr, ar, w);
        return 0;
    }
    if (0.0 <= al) { out = fl; return 0; }
    if (0.0 >= ar) { out = fr; return 0; }
    if (0.0 <= as) { out = star(ul, fl, pl, al, 0.0); return 0; }
    out = star(ur, fr, pr, ar, 0.0);
    return 0;
}

inline double plm(double yl, double y0, double yr, double theta)
{
    double a = (y0 - yl) / (1.0 - 0.0) * theta;
    double b = (yr - yl) / (2.0 - 0.0);
    double c = (yr - y0) / (2.0 - 1.0) * theta;
    double sa = std::copysign(1.0, a), sb = std::copysign(1.0, b), sc = std::copysign(1.0, c);
    return 0.25 * std::abs(sa + sb) * (sa + sc) * std::min(std::min(std::abs(a), std::abs(b)), std::abs(c));
}

// component k of a primitive (rho, u1, u2, u3, p)
inline double get(const Prim& p, int k) { return k == 0 ? p.rho : k == 1 ? p.u1 : k == 2 ? p.u2 : k == 3 ? p.u3 : p.p; }
inline void put(Prim& p, int k, double v)
{
    if (k == 0) p.rho = v; else if (k == 1) p.u1 = v; else if (k == 2) p.u2 = v; else if (k == 3) p.u3 = v; else p.p = v;
}

} // namespace srhd
} // namespace oracle
