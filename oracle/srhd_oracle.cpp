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
#include "srhd_common.hpp"

namespace {

using namespace oracle::srhd;

// One forward-Euler stage of the 2D Cartesian SRHD scheme composed from the
// reference's physics (the reference has no such scheme): recover_primitive
// per cell, generalised-minmod slopes of (rho, u1, u2, u3, p), face states
// p -/+ g/2 (the minidisk pattern, minidisk_scheme.cpp:238-240), HLLE fluxes
// (physics_srhd.hpp:489-497), u1 = u - (dFx + dFy) dt / dl. Zero-gradient
// boundaries (ghost cells copy the edge cell). u, out: [4][N][N] (D, S1, S2, tau).
int tube_stage(int N, const double* u, double* out, double dt, double dl, double theta, double gm, double floor_,
               const double* avg, std::vector<Prim>& P, bool hllc = false, int64_t* rejected = nullptr)
{
    const size_t NN = size_t(N) * N;
    int bad = 0;
    for (size_t c = 0; c < NN; ++c)
    {
        double z[5] = {u[c], u[NN + c], u[2 * NN + c], 0.0, u[3 * NN + c]};
        int it = 0;
        bad += recover_primitive(z, gm, floor_, 0.0, P[c], it) != 0;
    }
    auto at = [&] (int i, int j) -> const Prim& {
        i = std::min(std::max(i, 0), N - 1);
        j = std::min(std::max(j, 0), N - 1);
        return P[size_t(i) * N + j];
    };
    auto state = [&] (int i, int j, int axis, double sign) {
        const Prim& l = axis == 0 ? at(i - 1, j) : at(i, j - 1);
        const Prim& c = at(i, j);
        const Prim& r = axis == 0 ? at(i + 1, j) : at(i, j + 1);
        Prim s;
        for (int k = 0; k < 5; ++k) put(s, k, get(c, k) + sign * (0.5 * plm(get(l, k), get(c, k), get(r, k), theta)));
        return s;
    };
    // face fluxes: x face (f, j) between cells (f-1, j) and (f, j), f in [0, N]
    // HLLC faces whose contact speed the reference would reject take the HLLE flux
    auto face = [&] (const Prim& l, const Prim& r, int axis, Cons& out_) {
        if (hllc && riemann(l, r, axis, gm, true, out_) == 0) return;
        if (hllc && rejected) ++*rejected;
        riemann(l, r, axis, gm, false, out_);
    };
    std::vector<Cons> fx(size_t(N + 1) * N), fy(size_t(N) * (N + 1));
    for (int f = 0; f <= N; ++f)
        for (int j = 0; j < N; ++j)
            face(state(f - 1, j, 0, +1.0), state(f, j, 0, -1.0), 1, fx[size_t(f) * N + j]);
    for (int i = 0; i < N; ++i)
        for (int f = 0; f <= N; ++f)
            face(state(i, f - 1, 1, +1.0), state(i, f, 1, -1.0), 2, fy[size_t(i) * (N + 1) + f]);
    const int comp[4] = {0, 1, 2, 4};
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j)
        {
            const size_t c = size_t(i) * N + j;
            for (int q = 0; q < 4; ++q)
            {
                const int k = comp[q];
                double dfx = fx[size_t(i + 1) * N + j].c[k] - fx[size_t(i) * N + j].c[k];
                double dfy = fy[size_t(i) * (N + 1) + j + 1].c[k] - fy[size_t(i) * (N + 1) + j].c[k];
                double v = u[q * NN + c] - (dfx + dfy) * dt / dl;
                if (avg) v = avg[q * NN + c] * 0.5 + v * (1 - 0.5);
                out[q * NN + c] = v;
            }
        }
    return bad;
}

// max over cells of the outer wavespeed magnitudes on both axes
double tube_max_speed(int N, const double* u, double gm, double floor_)
{
    const size_t NN = size_t(N) * N;
    double m = 0.0;
    for (size_t c = 0; c < NN; ++c)
    {
        double z[5] = {u[c], u[NN + c], u[2 * NN + c], 0.0, u[3 * NN + c]};
        Prim p;
        int it;
        recover_primitive(z, gm, floor_, 0.0, p, it);
        for (int axis = 1; axis <= 2; ++axis)
        {
            double am, ap;
            outer_wavespeeds(p, axis, gm, am, ap);
            m = std::max(m, std::max(std::abs(am), std::abs(ap)));
        }
    }
    return m;
}

} // namespace

extern "C" {

// Relativistic shock tube on the unit square: (rho, p) = (rho_l, p_l) where
// (x - 1/2) cos(angle) + (y - 1/2) sin(angle) < 0, else (rho_r, p_r); v = 0.
// Cell centres x_i = (i + 1/2) / N. u: [4][N][N] (D, S1, S2, tau).
void oracle_srhd_tube_initial(int32_t N, double angle, double rho_l, double p_l, double rho_r, double p_r,
                              double gamma_law_index, double* u)
{
    const size_t NN = size_t(N) * N;
    const double c = std::cos(angle), s = std::sin(angle);
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j)
        {
            const double x = (i + 0.5) / N, y = (j + 0.5) / N;
            const bool left = (x - 0.5) * c + (y - 0.5) * s < 0.0;
            Prim p{left ? rho_l : rho_r, 0.0, 0.0, 0.0, left ? p_l : p_r};
            Cons w = conserved_density(p, gamma_law_index);
            const size_t k = size_t(i) * N + j;
            u[k] = w.c[0]; u[NN + k] = w.c[1]; u[2 * NN + k] = w.c[2]; u[3 * NN + k] = w.c[4];
        }
}

// `steps` RK2 steps (advance_runge_kutta order 2); dt = cfl * dl / max speed
// of the step's initial state. Returns the final time; *failures counts
// zones whose recovery failed (status != 0).
// The same with the Riemann solver chosen: hllc = 0 HLLE, 1 HLLC; *rejected
// (nullable) counts HLLC faces that fell back to HLLE.
double oracle_srhd_tube_advance_solver(int32_t N, double* u, double time, int32_t steps, double cfl, double theta,
                                       double gamma_law_index, double temperature_floor, int32_t hllc,
                                       int64_t* failures, int64_t* rejected)
{
    const size_t NN = size_t(N) * N;
    const double dl = 1.0 / N;
    std::vector<double> u1(4 * NN), u2(4 * NN);
    std::vector<Prim> P(NN);
    int64_t bad = 0;
    if (rejected) *rejected = 0;
    for (int s = 0; s < steps; ++s)
    {
        const double dt = cfl * dl / tube_max_speed(N, u, gamma_law_index, temperature_floor);
        bad += tube_stage(N, u, u1.data(), dt, dl, theta, gamma_law_index, temperature_floor, nullptr, P, hllc != 0,
                          rejected);
        bad += tube_stage(N, u1.data(), u, dt, dl, theta, gamma_law_index, temperature_floor, u, P, hllc != 0,
                          rejected);
        const double t2 = (time + dt) + dt;
        time = time * 0.5 + t2 * (1 - 0.5);
    }
    if (failures) *failures = bad;
    return time;
}

double oracle_srhd_tube_advance(int32_t N, double* u, double time, int32_t steps, double cfl, double theta,
                                double gamma_law_index, double temperature_floor, int64_t* failures)
{
    return oracle_srhd_tube_advance_solver(N, u, time, steps, cfl, theta, gamma_law_index, temperature_floor, 0,
                                           failures, nullptr);
}

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
