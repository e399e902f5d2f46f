// ORACLE — test infrastructure only (see oracle_common.hpp).
//
// CPU restatement of the reference's special-relativistic hydrodynamics
// (src/physics_srhd.hpp), c = 1:
//   recover_primitive     :231-285  Newton on p, 50+1 iterations, |f| < 1e-12
//                                   (1e-8 on the last iteration)
//   conserved_density     :291-304
//   flux                  :310-324
//   outer_wavespeeds      :182-195
//   riemann_solver        :377-487  (HLLE and HLLC, Mignone & Bodo 2005)
// Arithmetic keeps the reference's evaluation order. The recovery also
// reports its iteration count and accepts an optional starting pressure (the
// reference always starts from p = 0).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include "oracle_common.hpp"

namespace {

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
int recover_primitive(const double* u, double gm, double temperature_floor, double p_start,
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

// riemann_solver (physics_srhd.hpp:377-487) in the fixed-face HLLE / HLLC modes.
int riemann(const Prim& pl, const Prim& pr, int axis, double gm, bool hllc, Cons& out)
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

    auto star = [&] (const Cons& u, const Cons& f, const Prim& p, double s) {
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
        for (int k = 0; k < 5; ++k) fs.c[k] = (f.c[k] + s * (us.c[k] - u.c[k])) - 0.0 * us.c[k];
        return fs;
    };
    if (0.0 <= al) { out = fl; return 0; }
    if (0.0 >= ar) { out = fr; return 0; }
    if (0.0 <= as) { out = star(ul, fl, pl, al); return 0; }
    out = star(ur, fr, pr, ar);
    return 0;
}

} // namespace

extern "C" {

// srhd::recover_primitive over n AoS zones (5 doubles each). p_start may be
// null (start from p = 0, as the reference does) or hold one start pressure
// per zone. iterations/status may be null.
void oracle_srhd_recover_primitive(const double* u, int64_t n, double gamma_law_index, double temperature_floor,
                                   const double* p_start, double* prim, int32_t* iterations, int32_t* status)
{
    for (int64_t i = 0; i < n; ++i)
    {
        Prim p{0, 0, 0, 0, 0};
        int it = 0;
        int s = recover_primitive(u + 5 * i, gamma_law_index, temperature_floor, p_start ? p_start[i] : 0.0, p, it);
        if (s != 0) p = Prim{0, 0, 0, 0, 0};
        prim[5 * i] = p.rho; prim[5 * i + 1] = p.u1; prim[5 * i + 2] = p.u2; prim[5 * i + 3] = p.u3; prim[5 * i + 4] = p.p;
        if (iterations) iterations[i] = it;
        if (status) status[i] = s;
    }
}

void oracle_srhd_conserved_density(const double* prim, int64_t n, double gamma_law_index, double* u)
{
    for (int64_t i = 0; i < n; ++i)
    {
        Cons c = conserved_density(load_prim(prim + 5 * i), gamma_law_index);
        for (int k = 0; k < 5; ++k) u[5 * i + k] = c.c[k];
    }
}

// HLLE (hllc = 0) or HLLC (hllc = 1) fluxes on n faces; axis in {1, 2, 3}.
// Returns the number of faces whose contact speed was rejected (the reference throws).
int64_t oracle_srhd_riemann(const double* pl, const double* pr, int64_t n, int32_t axis, double gamma_law_index,
                            int32_t hllc, double* f)
{
    int64_t bad = 0;
    for (int64_t i = 0; i < n; ++i)
    {
        Cons c{};
        bad += riemann(load_prim(pl + 5 * i), load_prim(pr + 5 * i), axis, gamma_law_index, hllc != 0, c);
        for (int k = 0; k < 5; ++k) f[5 * i + k] = c.c[k];
    }
    return bad;
}

// Seeded SRHD zone batch: rho log-uniform [rho_lo, rho_hi], p log-uniform
// [p_lo, p_hi], Lorentz factor log-uniform [1, w_hi] in an isotropic random
// direction (3 components). Writes primitives (5 per zone) and conserved.
void oracle_srhd_seeded_zones(uint64_t seed, int64_t n, double rho_lo, double rho_hi, double p_lo, double p_hi,
                              double w_hi, double gamma_law_index, double* prim, double* cons)
{
    for (int64_t i = 0; i < n; ++i)
    {
        uint64_t k = uint64_t(i) * 5;
        double r0 = oracle::uniform01(seed, k), r1 = oracle::uniform01(seed, k + 1), r2 = oracle::uniform01(seed, k + 2);
        double r3 = oracle::uniform01(seed, k + 3), r4 = oracle::uniform01(seed, k + 4);
        double rho = rho_lo * std::exp(r0 * std::log(rho_hi / rho_lo));
        double p = p_lo * std::exp(r1 * std::log(p_hi / p_lo));
        double W = std::exp(r2 * std::log(w_hi));
        double ub = std::sqrt(W * W - 1.0);
        double mu = 2.0 * r3 - 1.0;
        double ph = 2.0 * M_PI * r4;
        double st = std::sqrt(1.0 - mu * mu);
        Prim q{rho, ub * st * std::cos(ph), ub * st * std::sin(ph), ub * mu, p};
        double* o = prim + 5 * i;
        o[0] = q.rho; o[1] = q.u1; o[2] = q.u2; o[3] = q.u3; o[4] = q.p;
        Cons c = conserved_density(q, gamma_law_index);
        for (int m = 0; m < 5; ++m) cons[5 * i + m] = c.c[m];
    }
}

} // extern "C"
