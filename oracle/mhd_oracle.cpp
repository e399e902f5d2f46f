// ORACLE — test infrastructure only (see oracle_common.hpp).
//
// CPU restatement of the reference's constrained-transport ideal-MHD scheme
// on one periodic cube (src/scheme_mhd_v1.cpp:152-299 with
// local_periodic_boundary_extension, src/physics_mhd.hpp:216-390,
// src/mesh_cartesian_3d.hpp:236-305) and of the RK2 driver of
// examples/mhd3d.cpp:78-88,186-215 (each stage takes its own CFL dt; states
// and times are averaged with weighted_sum). Evaluation order follows the
// reference.
//
// Layouts (the reference's row-major nd arrays, last axis fastest):
//   uc  [N][N][N][5]   conserved (d, s1, s2, s3, e)
//   bf1 [N+1][N][N], bf2 [N][N+1][N], bf3 [N][N][N+1]   face-normal B
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include "oracle_common.hpp"

namespace {

struct V3 { double x[3]; };
struct Prim { double d, v[3], p, b[3]; };
struct Cons { double c[5]; };

inline double sum3(const double a[3], const double b[3])
{
    return ((0.0 + a[0] * b[0]) + a[1] * b[1]) + a[2] * b[2];
}

inline V3 cross(const double a[3], const double b[3])
{
    return V3{{a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]}};
}

// physics_mhd.hpp:290-303 (status instead of throw)
inline int recover_primitive(const Cons& u, const double b[3], double gm, Prim& p)
{
    const double d = u.c[0];
    const double S[3] = {u.c[1], u.c[2], u.c[3]};
    const double kinetic = 0.5 * sum3(S, S) / d;
    const double magnetic = 0.5 * sum3(b, b);
    const double pg = (u.c[4] - kinetic - magnetic) * (gm - 1);
    p.d = d;
    for (int k = 0; k < 3; ++k) { p.v[k] = S[k] / d; p.b[k] = b[k]; }
    p.p = pg;
    if (d < 0.0) return 1;
    if (pg < 0.0) return 2;
    return 0;
}

// physics_mhd.hpp:305-318
inline Cons conserved_density(const Prim& p, double gm)
{
    const double E = 0.5 * p.d * sum3(p.v, p.v) + p.p / (gm - 1.0) + 0.5 * sum3(p.b, p.b);
    return Cons{{p.d, p.d * p.v[0], p.d * p.v[1], p.d * p.v[2], E}};
}

// physics_mhd.hpp:324-347 for the unit normal of `axis` (0, 1, 2)
inline Cons flux(const Prim& p, int axis, double gm)
{
    const double n[3] = {double(axis == 0), double(axis == 1), double(axis == 2)};
    const double bn = sum3(p.b, n);
    const double vn = sum3(p.v, n);
    const double pt = p.p + 0.5 * sum3(p.b, p.b);
    const double pressure[5] = {0.0, pt * n[0], pt * n[1], pt * n[2], pt * vn};
    const double maxwell[5] = {0.0, -bn * p.b[0], -bn * p.b[1], -bn * p.b[2], -bn * sum3(p.b, p.v)};
    Cons u = conserved_density(p, gm);
    Cons f;
    for (int k = 0; k < 5; ++k) f.c[k] = vn * u.c[k] + pressure[k] + maxwell[k];
    return f;
}

// induction = cross(n, -cross(v, B)) (physics_mhd.hpp:177-180, 349-352)
inline V3 induction(const Prim& p, int axis)
{
    const double n[3] = {double(axis == 0), double(axis == 1), double(axis == 2)};
    V3 vb = cross(p.v, p.b);
    const double E[3] = {-vb.x[0], -vb.x[1], -vb.x[2]};
    return cross(n, E);
}

// fast_speed_squared / outer_wavespeeds (physics_mhd.hpp:216-237)
inline void outer_wavespeeds(const Prim& p, int axis, double gm, double& am, double& ap)
{
    const double n[3] = {double(axis == 0), double(axis == 1), double(axis == 2)};
    const double cs2 = gm * p.p / p.d;
    const double va2 = sum3(p.b, p.b) / p.d;
    const double bn = sum3(p.b, n);
    const double van2 = std::pow(bn, 2.0) / p.d;
    const double cf2 = cs2 + va2;
    const double cg2 = std::sqrt(cf2 * cf2 - 4.0 * cs2 * van2);
    const double fast2 = 0.5 * (cf2 + cg2);
    const double vn = sum3(n, p.v);
    const double cf = std::sqrt(fast2);
    am = vn - cf;
    ap = vn + cf;
}

// physics_mhd.hpp:239-249
inline double fastest_speed(const Prim& p, double gm)
{
    double m[3], q[3];
    for (int a = 0; a < 3; ++a) outer_wavespeeds(p, a, gm, m[a], q[a]);
    return std::max(std::max(std::max(std::abs(m[0]), std::abs(q[0])), std::max(std::abs(m[1]), std::abs(q[1]))),
                    std::max(std::abs(m[2]), std::abs(q[2])));
}

// with_longitudinal_field (physics_mhd.hpp:162-173)
inline Prim with_longitudinal_field(Prim p, int axis, double bl)
{
    const double n[3] = {double(axis == 0), double(axis == 1), double(axis == 2)};
    const double bdn = sum3(p.b, n);
    double b[3];
    for (int k = 0; k < 3; ++k) b[k] = (p.b[k] - bdn * n[k]) + bl * n[k];
    for (int k = 0; k < 3; ++k) p.b[k] = b[k];
    return p;
}

// riemann_hlle (physics_mhd.hpp:358-390): flux and E-field
inline void riemann_hlle(Prim pl, Prim pr, double bl, int axis, double gm, Cons& F, V3& E)
{
    pl = with_longitudinal_field(pl, axis, bl);
    pr = with_longitudinal_field(pr, axis, bl);
    const Cons ul = conserved_density(pl, gm), ur = conserved_density(pr, gm);
    const Cons fl = flux(pl, axis, gm), fr = flux(pr, axis, gm);
    const V3 il = induction(pl, axis), ir = induction(pr, axis);
    double alm, alp, arm, arp;
    outer_wavespeeds(pl, axis, gm, alm, alp);
    outer_wavespeeds(pr, axis, gm, arm, arp);
    const double ap = std::max(0.0, std::max(alp, arp));
    const double am = std::min(0.0, std::min(alm, arm));
    for (int k = 0; k < 5; ++k)
        F.c[k] = (ap * fl.c[k] - am * fr.c[k] - (ul.c[k] - ur.c[k]) * ap * am) / (ap - am);
    double hi[3];
    for (int k = 0; k < 3; ++k)
        hi[k] = (ap * il.x[k] - am * ir.x[k] - (pl.b[k] - pr.b[k]) * ap * am) / (ap - am);
    const double n[3] = {double(axis == 0), double(axis == 1), double(axis == 2)};
    V3 c = cross(n, hi);
    for (int k = 0; k < 3; ++k) E.x[k] = -c.x[k];
}

inline double plm(double yl, double y0, double yr, double theta)
{
    double a = (y0 - yl) / (1.0 - 0.0) * theta;
    double b = (yr - yl) / (2.0 - 0.0);
    double c = (yr - y0) / (2.0 - 1.0) * theta;
    double sa = std::copysign(1.0, a), sb = std::copysign(1.0, b), sc = std::copysign(1.0, c);
    return 0.25 * std::abs(sa + sb) * (sa + sc) * std::min(std::min(std::abs(a), std::abs(b)), std::abs(c));
}

inline void prim_to_array(const Prim& p, double a[8])
{
    a[0] = p.d; a[1] = p.v[0]; a[2] = p.v[1]; a[3] = p.v[2]; a[4] = p.p; a[5] = p.b[0]; a[6] = p.b[1]; a[7] = p.b[2];
}

inline Prim array_to_prim(const double a[8])
{
    Prim p;
    p.d = a[0]; p.v[0] = a[1]; p.v[1] = a[2]; p.v[2] = a[3]; p.p = a[4]; p.b[0] = a[5]; p.b[1] = a[6]; p.b[2] = a[7];
    return p;
}

struct Mesh
{
    int N;
    int w(int i) const { return ((i % N) + N) % N; }
    size_t cell(int i, int j, int k) const { return (size_t(w(i)) * N + w(j)) * N + w(k); }
    // face-normal arrays of the reference's shapes, periodic image index
    size_t f1(int i, int j, int k) const { return (size_t(w(i)) * N + w(j)) * N + w(k); }   // [N+1][N][N], i<N
    size_t f2(int i, int j, int k) const { return (size_t(w(i)) * (N + 1) + w(j)) * N + w(k); }
    size_t f3(int i, int j, int k) const { return (size_t(w(i)) * N + w(j)) * (N + 1) + w(k); }
};

// One advance_mhd_ct (scheme_mhd_v1.cpp:265-299). Returns dt; status != 0 if
// a primitive recovery failed.
// Every loop runs its outer index on `threads` workers; each cell's
// arithmetic is the same as in a serial loop and the wavespeed maximum does
// not depend on the order, so the result does not depend on `threads`.
double advance_ct(int N, const double* uc, const double* bf1, const double* bf2, const double* bf3,
                  double dl, double cfl, double theta, double gm,
                  double* uc_out, double* bf1_out, double* bf2_out, double* bf3_out, int& status, int threads = 1)
{
    Mesh M{N};
    const size_t NN = size_t(N) * N * N;
    std::vector<double> P(NN * 8);
    std::vector<double> amax_row(N, 0.0);
    std::vector<int> status_row(N, 0);
    // primitive_array: face_to_cell then recover_primitive
    oracle::parallel_for(N, threads, [&] (int i) {
        double& amax = amax_row[i];
        int& status = status_row[i];
        for (int j = 0; j < N; ++j)
            for (int k = 0; k < N; ++k)
            {
                size_t c = M.cell(i, j, k);
                double b[3] = {0.5 * (bf1[(size_t(i) * N + j) * N + k] + bf1[(size_t(i + 1) * N + j) * N + k]),
                               0.5 * (bf2[(size_t(i) * (N + 1) + j) * N + k] + bf2[(size_t(i) * (N + 1) + j + 1) * N + k]),
                               0.5 * (bf3[(size_t(i) * N + j) * (N + 1) + k] + bf3[(size_t(i) * N + j) * (N + 1) + k + 1])};
                Cons u;
                for (int q = 0; q < 5; ++q) u.c[q] = uc[c * 5 + q];
                Prim p;
                status |= recover_primitive(u, b, gm, p);
                prim_to_array(p, &P[c * 8]);
                amax = std::max(amax, fastest_speed(p, gm));
            }
    });
    status = 0;
    double amax = 0.0;
    for (int i = 0; i < N; ++i)
    {
        status |= status_row[i];
        amax = std::max(amax, amax_row[i]);
    }
    // face fluxes and E-fields on the N+1 layers of each face array (the
    // reference's flux_arrays shapes): face (i,j,k) of axis a lies between
    // cell (i,j,k) - e_a and cell (i,j,k) (cells periodic); its normal field
    // is the face array's own layer, so layer N uses bf[N], not bf[0].
    auto fsize = [N] (int a) { return size_t(N + (a == 0)) * (N + (a == 1)) * (N + (a == 2)); };
    auto fid = [N] (int a, int i, int j, int k) {
        return (size_t(i) * (N + (a == 1)) + j) * (N + (a == 2)) + k;
    };
    std::vector<double> F[3], E[3];
    for (int a = 0; a < 3; ++a)
    {
        F[a].resize(fsize(a) * 5);
        E[a].resize(fsize(a) * 3);
        const double* bfa = a == 0 ? bf1 : (a == 1 ? bf2 : bf3);
        oracle::parallel_for(N + (a == 0), threads, [&] (int i) {
            for (int j = 0; j < N + (a == 1); ++j)
                for (int k = 0; k < N + (a == 2); ++k)
                {
                    int di = a == 0, dj = a == 1, dk = a == 2;
                    double pm2[8], pm1[8], p0[8], p1[8];
                    std::memcpy(pm2, &P[M.cell(i - 2 * di, j - 2 * dj, k - 2 * dk) * 8], sizeof pm2);
                    std::memcpy(pm1, &P[M.cell(i - di, j - dj, k - dk) * 8], sizeof pm1);
                    std::memcpy(p0, &P[M.cell(i, j, k) * 8], sizeof p0);
                    std::memcpy(p1, &P[M.cell(i + di, j + dj, k + dk) * 8], sizeof p1);
                    double L[8], R[8];
                    for (int q = 0; q < 8; ++q)
                    {
                        double gl = plm(pm2[q], pm1[q], p0[q], theta);
                        double gr = plm(pm1[q], p0[q], p1[q], theta);
                        L[q] = pm1[q] + 0.5 * gl;
                        R[q] = p0[q] - 0.5 * gr;
                    }
                    Cons f;
                    V3 e;
                    riemann_hlle(array_to_prim(L), array_to_prim(R), bfa[fid(a, i, j, k)], a, gm, f, e);
                    const size_t id = fid(a, i, j, k);
                    for (int q = 0; q < 5; ++q) F[a][id * 5 + q] = f.c[q];
                    for (int q = 0; q < 3; ++q) E[a][id * 3 + q] = e.x[q];
                }
        });
    }
    // E of face array a at layer index n (no wrap) and transverse cells (wrapped)
    auto ef = [&] (int a, int comp, int i, int j, int k) {
        if (a != 0) i = M.w(i);
        if (a != 1) j = M.w(j);
        if (a != 2) k = M.w(k);
        return E[a][fid(a, i, j, k) * 3 + comp];
    };
    // edge_emf_from_face (scheme_mhd_v1.cpp:76-98); edge of axis a at
    // (i,j,k) spans from corner (i,j,k) along a.
    auto ee1 = [&] (int i, int j, int k) {
        double a = 0.5 * (ef(1, 0, i, j, k - 1) + ef(1, 0, i, j, k));   // ef2 | c1 | adjacent_mean(2)
        double b = 0.5 * (ef(2, 0, i, j - 1, k) + ef(2, 0, i, j, k));   // ef3 | c1 | adjacent_mean(1)
        return 0.5 * (a + b);
    };
    auto ee2 = [&] (int i, int j, int k) {
        double a = 0.5 * (ef(2, 1, i - 1, j, k) + ef(2, 1, i, j, k));   // ef3 | c2 | adjacent_mean(0)
        double b = 0.5 * (ef(0, 1, i, j, k - 1) + ef(0, 1, i, j, k));   // ef1 | c2 | adjacent_mean(2)
        return 0.5 * (a + b);
    };
    auto ee3 = [&] (int i, int j, int k) {
        double a = 0.5 * (ef(0, 2, i, j - 1, k) + ef(0, 2, i, j, k));   // ef1 | c3 | adjacent_mean(1)
        double b = 0.5 * (ef(1, 2, i - 1, j, k) + ef(1, 2, i, j, k));   // ef2 | c3 | adjacent_mean(0)
        return 0.5 * (a + b);
    };
    const double dt = cfl * dl / amax;
    oracle::parallel_for(N, threads, [&] (int i) {
        for (int j = 0; j < N; ++j)
            for (int k = 0; k < N; ++k)
            {
                size_t c = M.cell(i, j, k);
                for (int q = 0; q < 5; ++q)
                {
                    double d1 = F[0][fid(0, i + 1, j, k) * 5 + q] - F[0][fid(0, i, j, k) * 5 + q];
                    double d2 = F[1][fid(1, i, j + 1, k) * 5 + q] - F[1][fid(1, i, j, k) * 5 + q];
                    double d3 = F[2][fid(2, i, j, k + 1) * 5 + q] - F[2][fid(2, i, j, k) * 5 + q];
                    double dc = d1 + d2 + d3;
                    uc_out[c * 5 + q] = uc[c * 5 + q] - dc * dt / dl;
                }
            }
    });
    // solenoidal_difference: cf1 = d2(ee3) - d3(ee2), cf2 = d3(ee1) - d1(ee3), cf3 = d1(ee2) - d2(ee1)
    oracle::parallel_for(N + 1, threads, [&] (int i) {
        for (int j = 0; j < N; ++j)
            for (int k = 0; k < N; ++k)
            {
                double cf = (ee3(i, j + 1, k) - ee3(i, j, k)) - (ee2(i, j, k + 1) - ee2(i, j, k));
                size_t f = (size_t(i) * N + j) * N + k;
                bf1_out[f] = bf1[f] - cf * dt / dl;
            }
    });
    oracle::parallel_for(N, threads, [&] (int i) {
        for (int j = 0; j <= N; ++j)
            for (int k = 0; k < N; ++k)
            {
                double cf = (ee1(i, j, k + 1) - ee1(i, j, k)) - (ee3(i + 1, j, k) - ee3(i, j, k));
                size_t f = (size_t(i) * (N + 1) + j) * N + k;
                bf2_out[f] = bf2[f] - cf * dt / dl;
            }
    });
    oracle::parallel_for(N, threads, [&] (int i) {
        for (int j = 0; j < N; ++j)
            for (int k = 0; k <= N; ++k)
            {
                double cf = (ee2(i + 1, j, k) - ee2(i, j, k)) - (ee1(i, j + 1, k) - ee1(i, j, k));
                size_t f = (size_t(i) * N + j) * (N + 1) + k;
                bf3_out[f] = bf3[f] - cf * dt / dl;
            }
    });
    return dt;
}

} // namespace

extern "C" {

// riemann_hlle on n face pairs; axis in {1, 2, 3}; out: flux (5) + E (3).
void oracle_mhd_riemann_hlle(const double* pl, const double* pr, const double* bl, int64_t n, uint32_t axis,
                             double gamma_law_index, double* out)
{
    for (int64_t i = 0; i < n; ++i)
    {
        Cons F;
        V3 E;
        riemann_hlle(array_to_prim(pl + 8 * i), array_to_prim(pr + 8 * i), bl[i], int(axis) - 1, gamma_law_index, F, E);
        for (int k = 0; k < 5; ++k) out[8 * i + k] = F.c[k];
        for (int k = 0; k < 3; ++k) out[8 * i + 5 + k] = E.x[k];
    }
}

// conserved_density then recover_primitive on n primitive 8-tuples; returns
// the number of zones whose recovery failed.
int64_t oracle_mhd_round_trip(const double* prim, int64_t n, double gm, double* cons, double* back)
{
    int64_t bad = 0;
    for (int64_t i = 0; i < n; ++i)
    {
        Prim p = array_to_prim(prim + 8 * i);
        Cons u = conserved_density(p, gm);
        for (int q = 0; q < 5; ++q) cons[5 * i + q] = u.c[q];
        Prim r;
        bad += recover_primitive(u, p.b, gm, r) != 0;
        prim_to_array(r, back + 8 * i);
    }
    return bad;
}

// One advance_mhd_ct step; returns dt (negative if a zone failed).
double oracle_mhd_advance_ct(int32_t N, const double* uc, const double* bf1, const double* bf2, const double* bf3,
                             double dl, double cfl, double plm_theta, double gamma_law_index,
                             double* uc_out, double* bf1_out, double* bf2_out, double* bf3_out)
{
    int status = 0;
    double dt = advance_ct(N, uc, bf1, bf2, bf3, dl, cfl, plm_theta, gamma_law_index, uc_out, bf1_out, bf2_out,
                           bf3_out, status);
    return status ? -1.0 : dt;
}

// `steps` RK2 steps of examples/mhd3d.cpp (advance_runge_kutta order 2 over
// advance_mhd_ct); arrays updated in place; returns the final time.
double oracle_mhd_rk2_threads(int32_t N, double* uc, double* bf1, double* bf2, double* bf3, double time,
                              int32_t steps, double dl, double cfl, double plm_theta, double gamma_law_index,
                              int32_t threads);

double oracle_mhd_rk2(int32_t N, double* uc, double* bf1, double* bf2, double* bf3, double time, int32_t steps,
                      double dl, double cfl, double plm_theta, double gamma_law_index)
{
    return oracle_mhd_rk2_threads(N, uc, bf1, bf2, bf3, time, steps, dl, cfl, plm_theta, gamma_law_index, 1);
}

// The same on `threads` workers (same result for any thread count).
double oracle_mhd_rk2_threads(int32_t N, double* uc, double* bf1, double* bf2, double* bf3, double time,
                              int32_t steps, double dl, double cfl, double plm_theta, double gamma_law_index,
                              int32_t threads)
{
    const size_t nc = size_t(N) * N * N * 5, nf = size_t(N + 1) * N * N;
    std::vector<double> u1(nc), b11(nf), b21(nf), b31(nf), u2(nc), b12(nf), b22(nf), b32(nf);
    int status = 0;
    for (int s = 0; s < steps; ++s)
    {
        int s0 = 0, s1 = 0;
        double dt0 = advance_ct(N, uc, bf1, bf2, bf3, dl, cfl, plm_theta, gamma_law_index,
                                u1.data(), b11.data(), b21.data(), b31.data(), s0, threads);
        double t1 = time + dt0;
        double dt1 = advance_ct(N, u1.data(), b11.data(), b21.data(), b31.data(), dl, cfl, plm_theta, gamma_law_index,
                                u2.data(), b12.data(), b22.data(), b32.data(), s1, threads);
        status |= s0 | s1;
        double t2 = t1 + dt1;
        for (size_t q = 0; q < nc; ++q) uc[q] = uc[q] * 0.5 + u2[q] * (1 - 0.5);
        for (size_t q = 0; q < nf; ++q)
        {
            bf1[q] = bf1[q] * 0.5 + b12[q] * (1 - 0.5);
            bf2[q] = bf2[q] * 0.5 + b22[q] * (1 - 0.5);
            bf3[q] = bf3[q] * 0.5 + b32[q] * (1 - 0.5);
        }
        time = time * 0.5 + t2 * (1 - 0.5);
    }
    return status ? -1.0 : time;
}

// Seeded initial state of the MHD benchmark, discretised as
// mara::construct_conserved does (src/scheme_mhd_v1.cpp:311-342): vertices
// of the unit cube, the vector potential on cell edges, B.dA on faces from
// solenoidal_difference(A dl) / dA, cell-centred B by face_to_cell, then
// conserved_density of (rho = 1, v(x), p = 1, B). v and A are sums of
// `modes` Fourier modes (integer wavevectors 0 < |k| <= 4, random phases and
// transverse polarisations) from mara_mhd_mode_table; v_amp and a_amp scale them.
void oracle_mhd_initial(int32_t N, const double* table, int32_t modes, double v_amp, double a_amp,
                        double gamma_law_index, double* uc, double* bf1, double* bf2, double* bf3)
{
    const double dl = 1.0 / double(N);
    const double da = std::pow(dl, 2.0);
    auto lin = [N] (int i) { return 0.0 + (1.0 - 0.0) * double(i) / double(N + 1 - 1); };
    // table rows: kx ky kz phase_v vx vy vz phase_a ax ay az
    auto field = [&] (const double x[3], int which, double out[3]) {
        out[0] = out[1] = out[2] = 0.0;
        for (int m = 0; m < modes; ++m)
        {
            const double* t = table + 11 * m;
            const double arg = 2.0 * M_PI * (t[0] * x[0] + t[1] * x[1] + t[2] * x[2]) + (which == 0 ? t[3] : t[7]);
            const double s = std::sin(arg);
            for (int c = 0; c < 3; ++c) out[c] += (which == 0 ? t[4 + c] : t[8 + c]) * s;
        }
        const double amp = which == 0 ? v_amp : a_amp;
        for (int c = 0; c < 3; ++c) out[c] *= amp;
    };
    // edge values of A.dl
    auto ae = [&] (int axis, int i, int j, int k) {
        double x[3] = {lin(i), lin(j), lin(k)};
        if (axis == 0) x[0] = 0.5 * (lin(i) + lin(i + 1));
        if (axis == 1) x[1] = 0.5 * (lin(j) + lin(j + 1));
        if (axis == 2) x[2] = 0.5 * (lin(k) + lin(k + 1));
        double A[3];
        field(x, 1, A);
        return A[axis] * dl;
    };
    for (int i = 0; i <= N; ++i)
        for (int j = 0; j < N; ++j)
            for (int k = 0; k < N; ++k)
                bf1[(size_t(i) * N + j) * N + k] = ((ae(2, i, j + 1, k) - ae(2, i, j, k)) - (ae(1, i, j, k + 1) - ae(1, i, j, k))) / da;
    for (int i = 0; i < N; ++i)
        for (int j = 0; j <= N; ++j)
            for (int k = 0; k < N; ++k)
                bf2[(size_t(i) * (N + 1) + j) * N + k] = ((ae(0, i, j, k + 1) - ae(0, i, j, k)) - (ae(2, i + 1, j, k) - ae(2, i, j, k))) / da;
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j)
            for (int k = 0; k <= N; ++k)
                bf3[(size_t(i) * N + j) * (N + 1) + k] = ((ae(1, i + 1, j, k) - ae(1, i, j, k)) - (ae(0, i, j + 1, k) - ae(0, i, j, k))) / da;
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j)
            for (int k = 0; k < N; ++k)
            {
                double x[3] = {0.5 * (lin(i) + lin(i + 1)), 0.5 * (lin(j) + lin(j + 1)), 0.5 * (lin(k) + lin(k + 1))};
                Prim p;
                p.d = 1.0;
                field(x, 0, p.v);
                p.p = 1.0;
                p.b[0] = 0.5 * (bf1[(size_t(i) * N + j) * N + k] + bf1[(size_t(i + 1) * N + j) * N + k]);
                p.b[1] = 0.5 * (bf2[(size_t(i) * (N + 1) + j) * N + k] + bf2[(size_t(i) * (N + 1) + j + 1) * N + k]);
                p.b[2] = 0.5 * (bf3[(size_t(i) * N + j) * (N + 1) + k] + bf3[(size_t(i) * N + j) * (N + 1) + k + 1]);
                Cons u = conserved_density(p, gamma_law_index);
                for (int q = 0; q < 5; ++q) uc[((size_t(i) * N + j) * N + k) * 5 + q] = u.c[q];
            }
}

// The seeded Fourier-mode table of the MHD initial state (11 doubles per
// mode), the same recipe as the library's mara_mhd_mode_table, restated.
int oracle_mhd_mode_table(uint64_t seed, int32_t modes, double* table)
{
    uint64_t counter = 0;
    auto uni = [&] (uint64_t i) { return double(oracle::hash64(seed, i) >> 11) * 0x1.0p-53; };
    for (int m = 0; m < modes; ++m)
    {
        double k[3];
        for (int attempt = 0;; ++attempt)
        {
            for (int c = 0; c < 3; ++c) k[c] = double(int(oracle::hash64(seed, counter++) % 9) - 4);
            const double kk = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
            if (kk > 0.0 && kk <= 16.0) break;
            if (attempt > 10000) return 1;
        }
        const double kn = std::sqrt(k[0] * k[0] + k[1] * k[1] + k[2] * k[2]);
        auto unit = [&] (double out[3]) {
            const double mu = 2.0 * uni(counter++) - 1.0, ph = 2.0 * M_PI * uni(counter++);
            const double st = std::sqrt(1.0 - mu * mu);
            out[0] = st * std::cos(ph); out[1] = st * std::sin(ph); out[2] = mu;
        };
        double* t = table + 11 * m;
        t[0] = k[0]; t[1] = k[1]; t[2] = k[2];
        t[3] = 2.0 * M_PI * uni(counter++);
        unit(t + 4);
        t[7] = 2.0 * M_PI * uni(counter++);
        double r[3], a[3], norm2 = 0.0;
        do {
            unit(r);
            const double rk = (r[0] * k[0] + r[1] * k[1] + r[2] * k[2]) / (kn * kn);
            norm2 = 0.0;
            for (int c = 0; c < 3; ++c) { a[c] = r[c] - rk * k[c]; norm2 += a[c] * a[c]; }
        } while (norm2 < 1e-6);
        for (int c = 0; c < 3; ++c) t[8 + c] = a[c] / (std::sqrt(norm2) * kn);
    }
    return 0;
}

// max |div B| * dl over cells (divergence_difference of the face fluxes B.dA / dV).
double oracle_mhd_max_div_b(int32_t N, const double* bf1, const double* bf2, const double* bf3)
{
    double m = 0.0;
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j)
            for (int k = 0; k < N; ++k)
            {
                double d = (bf1[(size_t(i + 1) * N + j) * N + k] - bf1[(size_t(i) * N + j) * N + k])
                         + (bf2[(size_t(i) * (N + 1) + j + 1) * N + k] - bf2[(size_t(i) * (N + 1) + j) * N + k])
                         + (bf3[(size_t(i) * N + j) * (N + 1) + k + 1] - bf3[(size_t(i) * N + j) * (N + 1) + k]);
                m = std::max(m, std::abs(d));
            }
    return m;
}

} // extern "C"
