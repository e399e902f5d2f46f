// ORACLE — test infrastructure only (see oracle_common.hpp).
//
// CPU restatement of the reference's locally-isothermal binary-minidisk update:
//   problems/minidisk_scheme.cpp:294-355  minidisk::updated_conserved
//   problems/minidisk_scheme.cpp:222-288  godunov_and_viscous_fluxes
//   problems/minidisk_scheme.cpp:47-165   source fields, geometry, initial state
//   problems/minidisk.cpp:87-120          extend (halo-2 block, periodic wrap)
//   problems/minidisk.cpp:202-213         fixed-formula time step
//   src/physics_iso2d.hpp:99-182          iso2d primitive/flux/HLLE/sources
//   src/physics_two_body.hpp:54-218,395-444  binary orbit, potential, gravity
//   src/scheme_plm_gradient.hpp:44-70     generalised-minmod slope
//   src/app_control.hpp:178-183, src/mesh_amr.hpp:456-467  RK2 averaging
// Every arithmetic expression keeps the reference's evaluation order so that
// results agree to the last bit with the reference compiled by the same
// compiler (checked against the reference itself by tests/golden fixtures).
//
// Mesh layout used by the whole-grid entry points: structure-of-arrays,
// component-major [3][N][N], axis 0 = x (slow), axis 1 = y (contiguous),
// N = block_size << depth. Block (bi, bj) at level `depth` owns rows
// [bi*n, bi*n+n) and columns [bj*n, bj*n+n).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include "oracle_common.hpp"

extern "C" {

// Field-for-field the reference's minidisk::solver_data_t
// (problems/minidisk.hpp:77-93) plus the PLM theta that the reference
// hard-codes to 2.0 (problems/minidisk_scheme.cpp:313-314).
struct oracle_minidisk_params
{
    int32_t block_size;
    int32_t depth;
    double omega_frame;
    double mach_number;
    double nu;
    double domain_radius;
    double softening_length;
    double eccentricity;
    double mass_ratio;
    double sink_radius;
    double sink_rate;
    double buffer_rate;
    double buffer_scale;
    double cfl;
    double plm_theta;
};

}

namespace {

using P = oracle_minidisk_params;

struct V3 { double c[3]; };

// ---------------------------------------------------------------- two body
// physics_two_body.hpp:54-157 and 395-444 (G = 1, a = 1, M = 1).
struct PointMass { double mass, x, y, vx, vy; };

void binary_state(const P& sd, double t, PointMass& c1, PointMass& c2)
{
    const double G = 1.0, a = 1.0, M = 1.0;
    const double q = sd.mass_ratio, e = sd.eccentricity;
    const double W = std::sqrt(G * M / a / a / a);

    // eccentric_anomaly (physics_two_body.hpp:109-126)
    const double Mt = W * t;
    auto f = [e, Mt] (double E) { return E - e * std::sin(E) - Mt; };
    auto g = [e]     (double E) { return 1 - e * std::cos(E); };
    double E = Mt;
    while (std::abs(f(E)) > 1e-12) E -= f(E) / g(E);

    // orbital_state_from_eccentric_anomaly (physics_two_body.hpp:128-152)
    const double mu = q / (1.0 + q);
    const double M1 = M * (1.0 - mu);
    const double M2 = M * mu;
    const double x1  = -a * mu * (e - std::cos(E));
    const double y1  = +a * mu * (0 + std::sin(E)) * std::sqrt(1 - e * e);
    const double x2  = -x1 / q;
    const double y2  = -y1 / q;
    const double vx1 = -a * mu * W / (1 - e * std::cos(E)) * std::sin(E);
    const double vy1 = +a * mu * W / (1 - e * std::cos(E)) * std::cos(E) * std::sqrt(1 - e * e);
    const double vx2 = -vx1 / q;
    const double vy2 = -vy1 / q;

    // rotate(state, -omega_frame * t) via transform (physics_two_body.hpp:395-444)
    const double angle = -sd.omega_frame * t;
    const double cs = std::cos(-angle);
    const double sn = std::sin(-angle);
    auto rot = [cs, sn] (double m, double x, double y, double vx, double vy) {
        return PointMass{m,
            +x  * cs + y  * sn + 0.0,
            -x  * sn + y  * cs + 0.0,
            +vx * cs + vy * sn + 0.0,
            -vx * sn + vy * cs + 0.0};
    };
    c1 = rot(M1, x1, y1, vx1, vy1);
    c2 = rot(M2, x2, y2, vx2, vy2);
}

// physics_two_body.hpp:200-218
inline double potential(const PointMass& p, double x, double y, double rs)
{
    double dx = x - p.x, dy = y - p.y;
    double r2 = dx * dx + dy * dy;
    double s2 = std::pow(rs, 2.0);
    return -1.0 * p.mass / std::sqrt(r2 + s2);
}

inline void gravitational_acceleration(const PointMass& p, double x, double y, double rs, double& ax, double& ay)
{
    double dx = x - p.x, dy = y - p.y;
    double r2 = dx * dx + dy * dy;
    double s2 = std::pow(rs, 2.0);
    ax = -1.0 * p.mass / std::pow(r2 + s2, 1.5) * dx;
    ay = -1.0 * p.mass / std::pow(r2 + s2, 1.5) * dy;
}

// ---------------------------------------------------------------- geometry
// vertex_positions / cell_size (problems/minidisk_scheme.cpp:78-116)
inline double vertex(double R, int n, unsigned level, long b, int k)
{
    double dl = double(1 << level);
    double x0 = R * (-1 + 2 * b / dl);
    double x1 = R * (-1 + 2 * (b + 1) / dl);
    return x0 + (x1 - x0) * double(k) / double(n);   // nd::linspace(x0, x1, n + 1)
}

inline double center(double R, int n, unsigned level, long b, int k)
{
    return 0.5 * (vertex(R, n, level, b, k) + vertex(R, n, level, b, k + 1));  // adjacent_mean
}

inline double cell_size(const P& sd, unsigned level)
{
    return 2.0 * sd.domain_radius / double(sd.block_size) / double(1 << level);
}

// sound_speed_squared (problems/minidisk_scheme.cpp:127-132)
inline double sound_speed_squared(double x, double y, const P& sd)
{
    double ph = potential(PointMass{1.0, 0.0, 0.0, 0.0, 0.0}, x, y, sd.softening_length);
    return -ph / sd.mach_number / sd.mach_number;
}

// initial_primitive -> conserved_density (problems/minidisk_scheme.cpp:87-99)
inline V3 initial_primitive(double x, double y, const P& sd)
{
    double ph = potential(PointMass{1.0, 0.0, 0.0, 0.0, 0.0}, x, y, sd.softening_length);
    double r0 = std::sqrt(x * x + y * y);
    double vp = std::sqrt(-ph) - sd.omega_frame * r0;
    double vx = vp * (-y / r0);
    double vy = vp * ( x / r0);
    return V3{{1.0, vx, vy}};
}

inline V3 conserved_density(V3 p) { return V3{{p.c[0], p.c[0] * p.c[1], p.c[0] * p.c[2]}}; }
inline V3 recover_primitive(V3 u) { return V3{{u.c[0], u.c[1] / u.c[0], u.c[2] / u.c[0]}}; }

// ---------------------------------------------------------------- scheme
// scheme_plm_gradient.hpp:56-63 on unit coordinates (0, 1, 2)
inline double plm(double yl, double y0, double yr, double theta)
{
    double a = (y0 - yl) / (1.0 - 0.0) * theta;
    double b = (yr - yl) / (2.0 - 0.0);
    double c = (yr - y0) / (2.0 - 1.0) * theta;
    double sa = std::copysign(1.0, a), sb = std::copysign(1.0, b), sc = std::copysign(1.0, c);
    return 0.25 * std::abs(sa + sb) * (sa + sc) * std::min(std::min(std::abs(a), std::abs(b)), std::abs(c));
}

// iso2d::riemann_hlle (physics_iso2d.hpp:156-173); axis 0 -> nhat = x, 1 -> y
inline V3 riemann_hlle(V3 pl, V3 pr, double cs2, int axis)
{
    const double n1 = axis == 0 ? 1.0 : 0.0, n2 = axis == 0 ? 0.0 : 1.0;
    auto flux = [&] (V3 p) {
        double pg = p.c[0] * cs2;
        double vn = ((0.0 + n1 * p.c[1]) + n2 * p.c[2]) + 0.0 * 0.0;
        V3 u = conserved_density(p);
        return V3{{vn * u.c[0] + 0.0 * 0.0, vn * u.c[1] + pg * n1, vn * u.c[2] + pg * n2}};
    };
    V3 ul = conserved_density(pl), ur = conserved_density(pr);
    V3 fl = flux(pl), fr = flux(pr);
    double cs = std::sqrt(cs2);
    double vnl = ((0.0 + n1 * pl.c[1]) + n2 * pl.c[2]) + 0.0 * 0.0;
    double vnr = ((0.0 + n1 * pr.c[1]) + n2 * pr.c[2]) + 0.0 * 0.0;
    double alm = vnl - cs, alp = vnl + cs, arm = vnr - cs, arp = vnr + cs;
    double ap = std::max(0.0, std::max(alp, arp));
    double am = std::min(0.0, std::min(alm, arm));
    V3 f;
    for (int k = 0; k < 3; ++k)
        f.c[k] = (ap * fl.c[k] - am * fr.c[k] - (ul.c[k] - ur.c[k]) * ap * am) / (ap - am);
    return f;
}

// minidisk::updated_conserved for one block (problems/minidisk_scheme.cpp:294-355).
// uc: n*n AoS conserved; pe: (n+4)*(n+4) AoS primitive (halo 2); u1: n*n AoS out.
void updated_conserved_block(const P& sd, const V3* uc, const V3* pe, double time, double dt,
                             unsigned level, long bi, long bj, V3* u1, double theta)
{
    const int n = sd.block_size;
    const int ne = n + 4;
    const double R = sd.domain_radius;
    const double dl = cell_size(sd, level);
    auto PE = [&] (int i, int j) -> const V3& { return pe[i * ne + j]; };

    // estimate_gradient (problems/minidisk_scheme.cpp:213-216): gx (n+2)x(n+4), gy (n+4)x(n+2)
    std::vector<V3> gx((n + 2) * (n + 4)), gy((n + 4) * (n + 2));
    for (int i = 0; i < n + 2; ++i)
        for (int j = 0; j < n + 4; ++j)
            for (int k = 0; k < 3; ++k)
                gx[i * (n + 4) + j].c[k] = plm(PE(i, j).c[k], PE(i + 1, j).c[k], PE(i + 2, j).c[k], theta);
    for (int i = 0; i < n + 4; ++i)
        for (int j = 0; j < n + 2; ++j)
            for (int k = 0; k < 3; ++k)
                gy[i * (n + 2) + j].c[k] = plm(PE(i, j).c[k], PE(i, j + 1).c[k], PE(i, j + 2).c[k], theta);
    // gx(i, j) is the x-slope of pe(i+1, j); gy(i, j) the y-slope of pe(i, j+1).
    auto GX = [&] (int pi, int pj) -> const V3& { return gx[(pi - 1) * (n + 4) + pj]; };
    auto GY = [&] (int pi, int pj) -> const V3& { return gy[pi * (n + 2) + (pj - 1)]; };

    // godunov_and_viscous_fluxes (problems/minidisk_scheme.cpp:222-288)
    // x faces: (n+1) x n, face f lies between pe rows f+1 and f+2.
    std::vector<V3> fx((n + 1) * n), fy(n * (n + 1));
    const double nu = sd.nu;
    for (int axis = 0; axis < 2; ++axis)
    {
        const int nf0 = axis == 0 ? n + 1 : n;
        const int nf1 = axis == 0 ? n : n + 1;
        for (int f0 = 0; f0 < nf0; ++f0)
        {
            for (int f1 = 0; f1 < nf1; ++f1)
            {
                // cells left (a) and right (b) of the face, in pe indices
                int ai = axis == 0 ? f0 + 1 : f0 + 2, aj = axis == 0 ? f1 + 2 : f1 + 1;
                int bi_ = axis == 0 ? f0 + 2 : f0 + 2, bj_ = axis == 0 ? f1 + 2 : f1 + 2;
                const V3& pa = PE(ai, aj);
                const V3& pb = PE(bi_, bj_);
                const V3& ga = axis == 0 ? GX(ai, aj) : GY(ai, aj);   // longitudinal
                const V3& gb = axis == 0 ? GX(bi_, bj_) : GY(bi_, bj_);
                const V3& ta = axis == 0 ? GY(ai, aj) : GX(ai, aj);   // transverse
                const V3& tb = axis == 0 ? GY(bi_, bj_) : GX(bi_, bj_);
                V3 pr_, pl_;   // reference names: pr = (pc + g/2)[left], pl = (pc - g/2)[right]
                for (int k = 0; k < 3; ++k)
                {
                    pr_.c[k] = pa.c[k] + 0.5 * ga.c[k];
                    pl_.c[k] = pb.c[k] - 0.5 * gb.c[k];
                }
                // face_coordinates (problems/minidisk_scheme.cpp:134-151)
                double xf = axis == 0 ? vertex(R, n, level, bi, f0) : center(R, n, level, bi, f0);
                double yf = axis == 0 ? center(R, n, level, bj, f1) : vertex(R, n, level, bj, f1);
                double cs2 = sound_speed_squared(xf, yf, sd);
                V3 F = riemann_hlle(pr_, pl_, cs2, axis);

                if (nu != 0.0)
                {
                    double sl = pl_.c[0], sr = pr_.c[0];
                    double mu = nu * 0.5 * (sl + sr);
                    // adjacent_mean of the limited gradients, divided by the cell size
                    double dvx_long = 0.5 * (ga.c[1] + gb.c[1]) / dl;
                    double dvy_long = 0.5 * (ga.c[2] + gb.c[2]) / dl;
                    double dvx_tran = 0.5 * (ta.c[1] + tb.c[1]) / dl;
                    double dvy_tran = 0.5 * (ta.c[2] + tb.c[2]) / dl;
                    if (axis == 0)
                    {
                        double dx_vx = dvx_long, dy_vx = dvx_tran, dx_vy = dvy_long, dy_vy = dvy_tran;
                        double tauxx = mu * (dx_vx - dy_vy);
                        double tauxy = mu * (dx_vy + dy_vx);
                        F.c[0] = F.c[0] + 0.0;
                        F.c[1] = F.c[1] + -tauxx;
                        F.c[2] = F.c[2] + -tauxy;
                    }
                    else
                    {
                        double dx_vx = dvx_tran, dy_vx = dvx_long, dx_vy = dvy_tran, dy_vy = dvy_long;
                        double tauyx =  mu * (dx_vy + dy_vx);
                        double tauyy = -mu * (dx_vx - dy_vy);
                        F.c[0] = F.c[0] + 0.0;
                        F.c[1] = F.c[1] + -tauyx;
                        F.c[2] = F.c[2] + -tauyy;
                    }
                }
                (axis == 0 ? fx[f0 * n + f1] : fy[f0 * (n + 1) + f1]) = F;
            }
        }
    }

    PointMass s1, s2;
    binary_state(sd, time, s1, s2);
    const double s6 = std::pow(sd.sink_radius, 6.0);
    const double om = sd.omega_frame;

    for (int i = 0; i < n; ++i)
    {
        for (int j = 0; j < n; ++j)
        {
            const double x = center(R, n, level, bi, i);
            const double y = center(R, n, level, bj, j);
            const V3& pc = PE(i + 2, j + 2);
            const V3& u = uc[i * n + j];

            V3 dfx, dfy;
            for (int k = 0; k < 3; ++k)
            {
                dfx.c[k] = fx[(i + 1) * n + j].c[k] - fx[i * n + j].c[k];
                dfy.c[k] = fy[i * (n + 1) + j + 1].c[k] - fy[i * (n + 1) + j].c[k];
            }
            double ag1x, ag1y, ag2x, ag2y;
            gravitational_acceleration(s1, x, y, sd.softening_length, ag1x, ag1y);
            gravitational_acceleration(s2, x, y, sd.softening_length, ag2x, ag2y);
            double corx = 2.0 * om * pc.c[2];
            double cory = 2.0 * om * -pc.c[1];
            double cenx = om * om * x;
            double ceny = om * om * y;

            auto sink = [&] (const PointMass& s) {
                double dx = x - s.x, dy = y - s.y;
                double r6 = std::pow(0.0 + dx * dx + dy * dy, 3.0);
                return sd.sink_rate * std::exp(-r6 / s6);
            };
            double sr1 = sink(s1), sr2 = sink(s2);
            double rr = std::sqrt(0.0 + x * x + y * y);
            double br = 0.5 * sd.buffer_rate * (1.0 + std::tanh((rr - R) / sd.buffer_scale));
            V3 ui = conserved_density(initial_primitive(x, y, sd));
            const double sig = pc.c[0];

            V3 out;
            for (int k = 0; k < 3; ++k)
            {
                double sg1 = k == 0 ? 0.0 : (k == 1 ? sig * ag1x : sig * ag1y);
                double sg2 = k == 0 ? 0.0 : (k == 1 ? sig * ag2x : sig * ag2y);
                double sf1 = k == 0 ? 0.0 : (k == 1 ? sig * cenx : sig * ceny);
                double sf2 = k == 0 ? 0.0 : (k == 1 ? sig * corx : sig * cory);
                double ss1 = -u.c[k] * sr1;
                double ss2 = -u.c[k] * sr2;
                double sb = -(u.c[k] - ui.c[k]) * br;
                out.c[k] = u.c[k] - (dfx.c[k] + dfy.c[k]) * dt / dl
                         + (sg1 + sg2 + ss1 + ss2 + sf1 + sf2 + sb) * dt;
            }
            u1[i * n + j] = out;
        }
    }
}

inline size_t soa(int N, int c, long i, long j) { return (size_t(c) * N + size_t(i)) * N + size_t(j); }

// One forward-Euler substep over the whole mesh: recover_primitive_array per
// block, extend with periodic wrap (problems/minidisk.cpp:87-120), then
// updated_conserved per block (problems/minidisk.cpp:172-189).
void substep(const P& sd, const double* u, double* out, double t, double dt, int threads,
             int block_begin = 0, int block_count = -1)
{
    const int n = sd.block_size;
    const int nb = 1 << sd.depth;
    const int N = n * nb;
    const int ne = n + 4;
    if (block_count < 0) block_count = nb * nb - block_begin;
    oracle::parallel_for(block_count, threads, [&] (int k) {
        const int b = block_begin + k;
        long bi = b / nb, bj = b % nb;
        std::vector<V3> uc(n * n), pe(ne * ne), u1(n * n);
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j)
                for (int k = 0; k < 3; ++k)
                    uc[i * n + j].c[k] = u[soa(N, k, bi * n + i, bj * n + j)];
        for (int i = 0; i < ne; ++i)
        {
            for (int j = 0; j < ne; ++j)
            {
                long gi = (bi * n + i - 2 + N) % N;
                long gj = (bj * n + j - 2 + N) % N;
                V3 w{{u[soa(N, 0, gi, gj)], u[soa(N, 1, gi, gj)], u[soa(N, 2, gi, gj)]}};
                pe[i * ne + j] = recover_primitive(w);
            }
        }
        updated_conserved_block(sd, uc.data(), pe.data(), t, dt, sd.depth, bi, bj, u1.data(), sd.plm_theta);
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j)
                for (int k = 0; k < 3; ++k)
                    out[soa(N, k, bi * n + i, bj * n + j)] = u1[i * n + j].c[k];
    });
}

} // namespace

extern "C" {

// Binary state (both masses) at time t in the rotating frame:
// out = {m1, x1, y1, vx1, vy1, m2, x2, y2, vx2, vy2}.
void oracle_minidisk_binary(const oracle_minidisk_params* sd, double t, double* out)
{
    PointMass a, b;
    binary_state(*sd, t, a, b);
    double v[10] = {a.mass, a.x, a.y, a.vx, a.vy, b.mass, b.x, b.y, b.vx, b.vy};
    std::memcpy(out, v, sizeof v);
}

// minidisk::updated_conserved on one block, AoS buffers as the reference holds them.
void oracle_minidisk_updated_conserved(const oracle_minidisk_params* sd, const double* uc, const double* pe,
                                       double time, double dt, uint32_t level, int64_t bi, int64_t bj, double* u1)
{
    updated_conserved_block(*sd, reinterpret_cast<const V3*>(uc), reinterpret_cast<const V3*>(pe),
                            time, dt, level, long(bi), long(bj), reinterpret_cast<V3*>(u1), sd->plm_theta);
}

// minidisk::estimate_gradient (problems/minidisk_scheme.cpp:213-216) on an AoS
// primitive array of shape (n0, n1): axis 0 -> (n0-2, n1), axis 1 -> (n0, n1-2).
void oracle_minidisk_estimate_gradient(const double* pc, int64_t n0, int64_t n1, int32_t axis, double theta, double* out)
{
    const int64_t m0 = axis == 0 ? n0 - 2 : n0, m1 = axis == 0 ? n1 : n1 - 2;
    for (int64_t i = 0; i < m0; ++i)
        for (int64_t j = 0; j < m1; ++j)
            for (int k = 0; k < 3; ++k)
            {
                int64_t di = axis == 0 ? 1 : 0, dj = axis == 0 ? 0 : 1;
                double yl = pc[((i) * n1 + j) * 3 + k];
                double y0 = pc[((i + di) * n1 + j + dj) * 3 + k];
                double yr = pc[((i + 2 * di) * n1 + j + 2 * dj) * 3 + k];
                out[(i * m1 + j) * 3 + k] = plm(yl, y0, yr, theta);
            }
}

// iso2d::recover_primitive over `count` AoS cells.
void oracle_minidisk_recover_primitive(const double* u, int64_t count, double* p)
{
    for (int64_t i = 0; i < count; ++i)
    {
        V3 w = recover_primitive(V3{{u[3 * i], u[3 * i + 1], u[3 * i + 2]}});
        p[3 * i] = w.c[0]; p[3 * i + 1] = w.c[1]; p[3 * i + 2] = w.c[2];
    }
}

// Fixed-formula time step (problems/minidisk.cpp:204-206).
double oracle_minidisk_dt_formula(const oracle_minidisk_params* sd, double t)
{
    double dx = 2.0 * sd->domain_radius / double(sd->block_size) / double(1 << sd->depth);
    double vmax = std::sqrt(1.0 * 0.5 / sd->softening_length);
    double cfl = sd->cfl * std::min(1.0, 0.01 + t / 0.05);
    return dx / vmax * cfl;
}

// CFL time step from a max-wavespeed reduction, in the form of
// scheme_mhd_v1.cpp:287 (cfl * dl / max speed) with iso2d::fastest_wavespeed
// (physics_iso2d.hpp:108-116) at the cell-centre sound speed.
double oracle_minidisk_dt_cfl(const oracle_minidisk_params* sd, const double* u)
{
    const int n = sd->block_size, nb = 1 << sd->depth, N = n * nb;
    double amax = 0.0;
    for (long i = 0; i < N; ++i)
    {
        for (long j = 0; j < N; ++j)
        {
            double x = center(sd->domain_radius, n, sd->depth, i / n, int(i % n));
            double y = center(sd->domain_radius, n, sd->depth, j / n, int(j % n));
            V3 p = recover_primitive(V3{{u[soa(N, 0, i, j)], u[soa(N, 1, i, j)], u[soa(N, 2, i, j)]}});
            double cs = std::sqrt(sound_speed_squared(x, y, *sd));
            double a = std::max(std::max(std::abs(p.c[1] - cs), std::abs(p.c[1] + cs)),
                                std::max(std::abs(p.c[2] - cs), std::abs(p.c[2] + cs)));
            amax = std::max(amax, a);
        }
    }
    double dl = 2.0 * sd->domain_radius / double(n) / double(1 << sd->depth);
    return sd->cfl * dl / amax;
}

// Initial conserved state (problems/minidisk_scheme.cpp:182-191) with the
// seeded density perturbation sigma * (1 + amplitude * (2U - 1)) applied to
// the primitive density before conversion. amplitude = 0 gives the
// reference's unperturbed initial state.
void oracle_minidisk_initial_conserved(const oracle_minidisk_params* sd, uint64_t seed, double amplitude, double* u)
{
    const int n = sd->block_size, nb = 1 << sd->depth, N = n * nb;
    for (long i = 0; i < N; ++i)
    {
        for (long j = 0; j < N; ++j)
        {
            double x = center(sd->domain_radius, n, sd->depth, i / n, int(i % n));
            double y = center(sd->domain_radius, n, sd->depth, j / n, int(j % n));
            V3 p = initial_primitive(x, y, *sd);
            if (amplitude != 0.0)
            {
                double r = 2.0 * oracle::uniform01(seed, uint64_t(i) * N + j) - 1.0;
                p.c[0] = p.c[0] * (1.0 + amplitude * r);
            }
            V3 w = conserved_density(p);
            for (int k = 0; k < 3; ++k) u[soa(N, k, i, j)] = w.c[k];
        }
    }
}

// One forward-Euler substep over the whole SoA mesh at time t.
void oracle_minidisk_substep(const oracle_minidisk_params* sd, const double* u, double* out, double t, double dt, int32_t threads)
{
    substep(*sd, u, out, t, dt, threads);
}

// The same substep restricted to blocks [block_begin, block_begin + block_count)
// of the row-major block order (a bounded CPU sample of a large mesh; every
// block does the full per-block work of the reference's block task).
void oracle_minidisk_substep_blocks(const oracle_minidisk_params* sd, const double* u, double* out, double t,
                                    double dt, int32_t threads, int32_t block_begin, int32_t block_count)
{
    substep(*sd, u, out, t, dt, threads, block_begin, block_count);
}

// Advance `steps` steps of order rk_order (1 or 2), following
// control::advance_runge_kutta (src/app_control.hpp:178-183): stage 2 runs at
// the stage-1 time t+dt, then u = u0*b + u2*(1-b) with b = 1/2, and
// t = t0*b + t2*(1-b). dt_mode 0: fixed formula; 1: CFL reduction.
// Returns the final time; u is updated in place.
// The time-series rate vector of a state at time t (the sums that the
// minidisk driver lists as to do, problems/minidisk.cpp:69): the source-term
// fields of updated_conserved (problems/minidisk_scheme.cpp:47-76, 337-352;
// src/physics_two_body.hpp:200-218), each summed over all cells times the
// cell area. out[16]: sink mass rates (2), sink momentum rates (4), gas force
// on each body (4), buffer mass rate, disk mass, disk angular momentum,
// torques on each body (2) and power on the binary.
void oracle_minidisk_rates(const oracle_minidisk_params* sd, const double* u, double t, double* out)
{
    const int n = sd->block_size, nb = 1 << sd->depth, N = n * nb;
    const double R = sd->domain_radius;
    const double dl = cell_size(*sd, sd->depth);
    PointMass s1, s2;
    binary_state(*sd, t, s1, s2);
    const double s6 = std::pow(sd->sink_radius, 6.0);
    double acc[13] = {};
    for (long i = 0; i < N; ++i)
    {
        for (long j = 0; j < N; ++j)
        {
            const double x = center(R, n, sd->depth, i / n, int(i % n));
            const double y = center(R, n, sd->depth, j / n, int(j % n));
            const double w[3] = {u[soa(N, 0, i, j)], u[soa(N, 1, i, j)], u[soa(N, 2, i, j)]};
            auto sink = [&] (const PointMass& s) {
                double dx = x - s.x, dy = y - s.y;
                double r6 = std::pow(0.0 + dx * dx + dy * dy, 3.0);
                return sd->sink_rate * std::exp(-r6 / s6);
            };
            const double sr1 = sink(s1), sr2 = sink(s2);
            double a1x, a1y, a2x, a2y;
            gravitational_acceleration(s1, x, y, sd->softening_length, a1x, a1y);
            gravitational_acceleration(s2, x, y, sd->softening_length, a2x, a2y);
            const double rr = std::sqrt(0.0 + x * x + y * y);
            const double br = 0.5 * sd->buffer_rate * (1.0 + std::tanh((rr - R) / sd->buffer_scale));
            const double v[13] = {
                w[0] * sr1, w[0] * sr2, w[1] * sr1, w[2] * sr1, w[1] * sr2, w[2] * sr2,
                -w[0] * a1x, -w[0] * a1y, -w[0] * a2x, -w[0] * a2y,
                (1.0 - w[0]) * br, w[0], x * w[2] - y * w[1]};
            for (int k = 0; k < 13; ++k) acc[k] += v[k];
        }
    }
    for (int k = 0; k < 13; ++k) out[k] = acc[k] * (dl * dl);
    out[13] = s1.x * out[7] - s1.y * out[6];
    out[14] = s2.x * out[9] - s2.y * out[8];
    out[15] = (out[6] * s1.vx + out[7] * s1.vy) + (out[8] * s2.vx + out[9] * s2.vy);
}

double oracle_minidisk_advance(const oracle_minidisk_params* sd, double* u, double t, int32_t steps,
                               int32_t rk_order, int32_t dt_mode, int32_t threads)
{
    const int N = sd->block_size << sd->depth;
    const size_t len = size_t(3) * N * N;
    std::vector<double> u1(len), u2(len);
    for (int s = 0; s < steps; ++s)
    {
        double dt = dt_mode == 0 ? oracle_minidisk_dt_formula(sd, t) : oracle_minidisk_dt_cfl(sd, u);
        if (rk_order == 1)
        {
            substep(*sd, u, u1.data(), t, dt, threads);
            std::memcpy(u, u1.data(), len * sizeof(double));
            t = t + dt;
        }
        else
        {
            substep(*sd, u, u1.data(), t, dt, threads);
            double t1 = t + dt;
            substep(*sd, u1.data(), u2.data(), t1, dt, threads);
            double t2 = t1 + dt;
            const double b = 0.5;
            for (size_t k = 0; k < len; ++k) u[k] = u[k] * b + u2[k] * (1.0 - b);
            t = t * b + t2 * (1.0 - b);
        }
    }
    return t;
}

} // extern "C"
