// ORACLE — test infrastructure only (see oracle_common.hpp).
//
// C entry points around the reference's OWN compiled scheme and physics code.
// This file is compiled together with the reference's sources (read in place
// from the reference checkout by oracle/Makefile) into oracle/_ref/libref.so.
// It exists to pin the oracle restatement and to produce golden fixtures; it
// contains only marshalling between flat double buffers and the reference's
// nd::shared_array / numeric::tuple_t types, plus the reference's driver loop
// restated where the original translation unit cannot be built here
// (problems/minidisk.cpp needs HDF5 and MPI).
#include <array>
#include <cstdint>
#include <cstring>
#include <utility>
#include <vector>
#include "minidisk.hpp"
#include "parallel_thread_pool.hpp"
#include "physics_srhd.hpp"
#include "physics_two_body.hpp"
#include "scheme_mhd_v1.hpp"
#include "scheme_plm_gradient.hpp"
#include "scheme_sedov2d.hpp"
#include "ref_marshal.hpp"

namespace {

minidisk::solver_data_t solver_data(const double* v)
{
    // v = {block_size, depth, omega_frame, mach_number, nu, domain_radius,
    //      softening_length, eccentricity, mass_ratio, sink_radius, sink_rate,
    //      buffer_rate, buffer_scale, cfl}
    return minidisk::solver_data_t{
        int(v[0]), int(v[1]), v[2], v[3], v[4], v[5], v[6], v[7], v[8], v[9], v[10], v[11], v[12], v[13]};
}

mesh::block_index_t<2> block_index(unsigned long level, unsigned long bi, unsigned long bj)
{
    return mesh::block_index_t<2>{level, numeric::array(bi, bj)};
}

} // namespace

extern "C" {

// minidisk::updated_conserved on one block (problems/minidisk_scheme.cpp:294).
int ref_minidisk_updated_conserved(const double* sdv, const double* uc, const double* pe,
                                   double time, double dt, uint32_t level, uint64_t bi, uint64_t bj, double* u1)
{
    try {
        auto sd = solver_data(sdv);
        auto n = std::size_t(sd.block_size);
        auto ua = make_array2<iso2d::conserved_density_t>(uc, n, n);
        auto pa = make_array2<iso2d::primitive_t>(pe, n + 4, n + 4);
        auto r = minidisk::updated_conserved(ua, pa, time, dt, block_index(level, bi, bj), sd);
        read_array2(r, u1);
        return 0;
    } catch (...) {
        return 1;
    }
}

// minidisk::estimate_gradient (problems/minidisk_scheme.cpp:213) on an AoS
// primitive array of shape (n0, n1).
int ref_minidisk_estimate_gradient(const double* pc, uint64_t n0, uint64_t n1, uint32_t axis, double theta, double* out)
{
    auto pa = make_array2<iso2d::primitive_t>(pc, n0, n1);
    read_array2(minidisk::estimate_gradient(pa, axis, theta), out);
    return 0;
}

// One forward-Euler substep over a periodic uniform mesh of depth `depth`,
// SoA [3][N][N] in and out, one mara::ThreadPool task per block per phase,
// in the shape of problems/minidisk.cpp:172-189 (recover_primitive_array per
// block, extend from the 3x3 neighbours, updated_conserved per block).
int ref_minidisk_substep(const double* sdv, const double* u, double* out, double t, double dt, int32_t threads)
{
    auto sd = solver_data(sdv);
    const std::size_t n = sd.block_size, nb = std::size_t(1) << sd.depth, N = n * nb;
    auto pool = mara::ThreadPool(threads < 1 ? 1 : threads);

    std::vector<minidisk::primitive_array_t> pc(nb * nb);
    std::vector<minidisk::conserved_array_t> uc(nb * nb);
    {
        std::vector<std::future<int>> fut;
        for (std::size_t b = 0; b < nb * nb; ++b)
        {
            fut.push_back(pool.enqueue(0, [&, b] {
                std::size_t bi = b / nb, bj = b % nb;
                std::vector<double> buf(n * n * 3);
                for (std::size_t i = 0; i < n; ++i)
                    for (std::size_t j = 0; j < n; ++j)
                        for (int k = 0; k < 3; ++k)
                            buf[(i * n + j) * 3 + k] = u[(k * N + bi * n + i) * N + bj * n + j];
                uc[b] = make_array2<iso2d::conserved_density_t>(buf.data(), n, n);
                pc[b] = minidisk::recover_primitive_array(uc[b]);
                return 0;
            }));
        }
        for (auto& f : fut) f.get();
    }
    std::vector<std::future<int>> fut;
    for (std::size_t b = 0; b < nb * nb; ++b)
    {
        fut.push_back(pool.enqueue(0, [&, b] {
            std::size_t bi = b / nb, bj = b % nb;
            // extend (problems/minidisk.cpp:87-120): halo 2 from the 3x3 neighbours, periodic
            auto pe = nd::make_unique_array<iso2d::primitive_t, 2>(nd::uivec(n + 4, n + 4));
            for (std::size_t i = 0; i < n + 4; ++i)
            {
                for (std::size_t j = 0; j < n + 4; ++j)
                {
                    std::size_t ci = i < 2 ? (bi + nb - 1) % nb : (i >= n + 2 ? (bi + 1) % nb : bi);
                    std::size_t cj = j < 2 ? (bj + nb - 1) % nb : (j >= n + 2 ? (bj + 1) % nb : bj);
                    std::size_t ii = i < 2 ? i - 2 + n : (i >= n + 2 ? i - 2 - n : i - 2);
                    std::size_t jj = j < 2 ? j - 2 + n : (j >= n + 2 ? j - 2 - n : j - 2);
                    pe(i, j) = pc[ci * nb + cj](ii, jj);
                }
            }
            auto r = minidisk::updated_conserved(uc[b], nd::make_shared_array(std::move(pe)), t, dt,
                                                 block_index(sd.depth, bi, bj), sd);
            for (std::size_t i = 0; i < n; ++i)
                for (std::size_t j = 0; j < n; ++j)
                {
                    double v[3];
                    from_tuple(r(i, j), v);
                    for (int k = 0; k < 3; ++k) out[(k * N + bi * n + i) * N + bj * n + j] = v[k];
                }
            return 0;
        }));
    }
    for (auto& f : fut) f.get();
    return 0;
}

// Binary state in the rotating frame, as updated_conserved computes it
// (problems/minidisk_scheme.cpp:329-335): out = {m1,x1,y1,vx1,vy1,m2,x2,y2,vx2,vy2}.
void ref_minidisk_binary(double mass_ratio, double eccentricity, double omega_frame, double t, double* out)
{
    auto el = two_body::orbital_elements(1.0, 1.0, mass_ratio, eccentricity);
    auto s = two_body::rotate(two_body::orbital_state(el, t), -dimensional::unit_rate(omega_frame) * dimensional::unit_time(t));
    double v[10] = {s.first.mass.value, s.first.position_x.value, s.first.position_y.value,
                    s.first.velocity_x.value, s.first.velocity_y.value,
                    s.second.mass.value, s.second.position_x.value, s.second.position_y.value,
                    s.second.velocity_x.value, s.second.velocity_y.value};
    std::memcpy(out, v, sizeof v);
}

// srhd::recover_primitive (src/physics_srhd.hpp:231-285) over n AoS zones of 5;
// status[i] = 0 ok, 1 the reference threw.
void ref_srhd_recover_primitive(const double* u, int64_t n, double gamma_law_index, double temperature_floor,
                                double* p, int32_t* status)
{
    for (int64_t i = 0; i < n; ++i)
    {
        try {
            auto r = srhd::recover_primitive(to_tuple<srhd::conserved_density_t>(u + 5 * i), gamma_law_index, temperature_floor);
            from_tuple(r, p + 5 * i);
            status[i] = 0;
        } catch (...) {
            for (int k = 0; k < 5; ++k) p[5 * i + k] = 0.0;
            status[i] = 1;
        }
    }
}

// srhd::conserved_density (src/physics_srhd.hpp:291-304) over n zones.
void ref_srhd_conserved_density(const double* p, int64_t n, double gamma_law_index, double* u)
{
    for (int64_t i = 0; i < n; ++i)
        from_tuple(srhd::conserved_density(to_tuple<srhd::primitive_t>(p + 5 * i), gamma_law_index), u + 5 * i);
}

// srhd::riemann_hlle / riemann_hllc (src/physics_srhd.hpp:489-507) over n
// face pairs; axis in {1,2,3}; hllc != 0 selects HLLC.
int ref_srhd_riemann(const double* pl, const double* pr, int64_t n, uint32_t axis, double gamma_law_index,
                     int32_t hllc, double* f)
{
    try {
        auto nhat = geometric::unit_vector_on(axis);
        for (int64_t i = 0; i < n; ++i)
        {
            auto a = to_tuple<srhd::primitive_t>(pl + 5 * i);
            auto b = to_tuple<srhd::primitive_t>(pr + 5 * i);
            auto r = hllc ? srhd::riemann_hllc(a, b, nhat, gamma_law_index) : srhd::riemann_hlle(a, b, nhat, gamma_law_index);
            from_tuple(r, f + 5 * i);
        }
        return 0;
    } catch (...) {
        return 1;
    }
}

// mara::plm_gradient on unit coordinates (src/scheme_plm_gradient.hpp:44-70),
// on dimensional quantities as every scheme calls it (with raw doubles the
// reference's unqualified abs() would bind to the int overload).
double ref_plm_gradient(double theta, double yl, double y0, double yr)
{
    using q = dimensional::unit_scalar;
    return mara::plm_gradient_scalar_t<double>{0.0, 1.0, 2.0, theta}(numeric::tuple(q(yl), q(y0), q(yr))).value;
}

// mhd::riemann_hlle (src/physics_mhd.hpp:358-390) on n face pairs of 8
// primitives; axis in {1, 2, 3}; out: flux (5) then E-field (3) per face.
void ref_mhd_riemann_hlle(const double* pl, const double* pr, const double* bl, int64_t n, uint32_t axis,
                          double gamma_law_index, double* out)
{
    for (int64_t i = 0; i < n; ++i)
    {
        auto a = to_tuple<mhd::primitive_t>(pl + 8 * i);
        auto b = to_tuple<mhd::primitive_t>(pr + 8 * i);
        auto [f, e] = mhd::riemann_hlle(a, b, mhd::unit_magnetic_field(bl[i]), geometric::unit_vector_on(axis),
                                        gamma_law_index);
        from_tuple(f, out + 8 * i);
        out[8 * i + 5] = e.component_1().value;
        out[8 * i + 6] = e.component_2().value;
        out[8 * i + 7] = e.component_3().value;
    }
}

// iso2d pointwise physics (src/physics_iso2d.hpp:99-173) on n points with
// their local cs^2; axis in {1, 2}. Per point: flux(pl) [3], outer_wavespeeds(pl)
// [2], fastest_wavespeed(pl), riemann_hlle(pl, pr) [3].
void ref_iso2d_pointwise(const double* pl, const double* pr, const double* cs2, int64_t n, uint32_t axis,
                         double* flux, double* outer, double* fastest, double* hlle)
{
    const auto nhat = geometric::unit_vector_on(axis);
    for (int64_t i = 0; i < n; ++i)
    {
        const auto a = to_tuple<iso2d::primitive_t>(pl + 3 * i);
        const auto b = to_tuple<iso2d::primitive_t>(pr + 3 * i);
        const auto c2 = dimensional::unit_specific_energy(cs2[i]);
        from_tuple(iso2d::flux(a, nhat, c2), flux + 3 * i);
        const auto [wm, wp] = iso2d::outer_wavespeeds(a, nhat, c2);
        outer[2 * i] = wm.value;
        outer[2 * i + 1] = wp.value;
        fastest[i] = iso2d::fastest_wavespeed(a, c2).value;
        from_tuple(iso2d::riemann_hlle(a, b, c2, nhat), hlle + 3 * i);
    }
}

// mhd pointwise physics (src/physics_mhd.hpp:216-356) on n primitive
// 8-tuples; axis in {1, 2, 3}. Per point: flux [5], fast_speed_squared along
// the axis, fastest_speed.
void ref_mhd_pointwise(const double* p, int64_t n, uint32_t axis, double gamma_law_index, double* flux, double* cf2,
                       double* fastest)
{
    const auto nhat = geometric::unit_vector_on(axis);
    for (int64_t i = 0; i < n; ++i)
    {
        const auto a = to_tuple<mhd::primitive_t>(p + 8 * i);
        from_tuple(mhd::flux(a, nhat, gamma_law_index), flux + 5 * i);
        cf2[i] = mhd::fast_speed_squared(a, nhat, gamma_law_index).value;
        fastest[i] = mhd::fastest_speed(a, gamma_law_index).value;
    }
}

// mhd::recover_primitive (src/physics_mhd.hpp:290-303) of n conserved
// 5-tuples with cell fields b [n][3]; status 0, or 1 where it throws
// (negative density or pressure; the primitives are then left zero).
void ref_mhd_recover_primitive(const double* u, const double* b, int64_t n, double gamma_law_index, double* p,
                               int32_t* status)
{
    for (int64_t i = 0; i < n; ++i)
    {
        const auto c = to_tuple<mhd::conserved_density_t>(u + 5 * i);
        const auto bv = geometric::euclidean_vector(mhd::unit_magnetic_field(b[3 * i]),
                                                    mhd::unit_magnetic_field(b[3 * i + 1]),
                                                    mhd::unit_magnetic_field(b[3 * i + 2]));
        try {
            from_tuple(mhd::recover_primitive(c, bv, gamma_law_index), p + 8 * i);
            status[i] = 0;
        } catch (...) {
            for (int k = 0; k < 8; ++k) p[8 * i + k] = 0.0;
            status[i] = 1;
        }
    }
}

// mhd::conserved_density then mhd::recover_primitive (the round trip of
// test_mhd, src/physics_mhd.hpp:405-415) on n primitive 8-tuples.
int ref_mhd_round_trip(const double* prim, int64_t n, double gamma_law_index, double* cons, double* back)
{
    try {
        for (int64_t i = 0; i < n; ++i)
        {
            auto p = to_tuple<mhd::primitive_t>(prim + 8 * i);
            auto u = mhd::conserved_density(p, gamma_law_index);
            from_tuple(u, cons + 5 * i);
            from_tuple(mhd::recover_primitive(u, mhd::magnetic_field_vector(p), gamma_law_index), back + 8 * i);
        }
        return 0;
    } catch (...) {
        return 1;
    }
}

// mara::advance_mhd_ct (src/scheme_mhd_v1.cpp:265-299) on one periodic cube
// with local_periodic_boundary_extension. uc [N][N][N][5]; bf1 [N+1][N][N],
// bf2 [N][N+1][N], bf3 [N][N][N+1]. Returns t + dt, or -1 if it threw.
double ref_mhd_advance_ct(int32_t N, double time, const double* uc, const double* bf1, const double* bf2,
                          const double* bf3, double dl, double cfl, double plm_theta,
                          double* uc_out, double* bf1_out, double* bf2_out, double* bf3_out)
{
    try {
        using B = mhd::unit_magnetic_field;
        const std::size_t n = N;
        auto u = nd::make_unique_array<mhd::conserved_density_t, 3>(nd::uivec(n, n, n));
        for (std::size_t i = 0; i < n; ++i)
            for (std::size_t j = 0; j < n; ++j)
                for (std::size_t k = 0; k < n; ++k)
                    u(i, j, k) = to_tuple<mhd::conserved_density_t>(uc + ((i * n + j) * n + k) * 5);
        auto face = [&] (const double* src, std::size_t a, std::size_t b, std::size_t c) {
            auto f = nd::make_unique_array<B, 3>(nd::uivec(a, b, c));
            for (std::size_t i = 0; i < a; ++i)
                for (std::size_t j = 0; j < b; ++j)
                    for (std::size_t k = 0; k < c; ++k)
                        f(i, j, k) = B(src[(i * b + j) * c + k]);
            return nd::make_shared_array(std::move(f));
        };
        auto bc = mara::local_periodic_boundary_extension();
        auto [t1, u1, b1, b2, b3] = mara::advance_mhd_ct(time, nd::make_shared_array(std::move(u)),
                                                         face(bf1, n + 1, n, n), face(bf2, n, n + 1, n),
                                                         face(bf3, n, n, n + 1), dl, cfl, plm_theta, *bc);
        for (std::size_t i = 0; i < n; ++i)
            for (std::size_t j = 0; j < n; ++j)
                for (std::size_t k = 0; k < n; ++k)
                    from_tuple(u1(i, j, k), uc_out + ((i * n + j) * n + k) * 5);
        auto read = [] (const auto& f, double* dst) {
            std::size_t a = shape(f, 0), b = shape(f, 1), c = shape(f, 2);
            for (std::size_t i = 0; i < a; ++i)
                for (std::size_t j = 0; j < b; ++j)
                    for (std::size_t k = 0; k < c; ++k)
                        dst[(i * b + j) * c + k] = f(i, j, k).value;
        };
        read(b1, bf1_out);
        read(b2, bf2_out);
        read(b3, bf3_out);
        return t1.value;
    } catch (...) {
        return -1.0;
    }
}

// two_body::recover_orbital_elements (physics_two_body.hpp:284-379) of a
// state {m1, x1, y1, vx1, vy1, m2, x2, y2, vx2, vy2} at time t:
// out = {a, M, q, e, x_cm, y_cm, vx_cm, vy_cm, pomega, tau}; 1 if unbound.
int ref_two_body_elements(const double* s, double t, double* out)
{
    using namespace two_body;
    using namespace dimensional;
    point_mass_t c1{unit_mass(s[0]), unit_length(s[1]), unit_length(s[2]), unit_velocity(s[3]), unit_velocity(s[4])};
    point_mass_t c2{unit_mass(s[5]), unit_length(s[6]), unit_length(s[7]), unit_velocity(s[8]), unit_velocity(s[9])};
    try
    {
        auto p = recover_orbital_elements(orbital_state_t{c1, c2}, unit_time(t));
        auto el = numeric::get<0>(p);
        auto o = numeric::get<1>(p);
        double v[10] = {semimajor_axis(el).value, total_mass(el).value, mass_ratio(el).value, eccentricity(el).value,
                        numeric::get<0>(o).value, numeric::get<1>(o).value, numeric::get<2>(o).value,
                        numeric::get<3>(o).value, numeric::get<4>(o).value, numeric::get<5>(o).value};
        std::memcpy(out, v, sizeof v);
        return 0;
    }
    catch (const std::invalid_argument&)
    {
        return 1;
    }
}

// two_body::orbital_state (physics_two_body.hpp:128-157) for elements
// (a, M, q, e) at time t: out = {m1, x1, y1, vx1, vy1, m2, x2, y2, vx2, vy2}.
void ref_two_body_state(double a, double M, double q, double e, double t, double* out)
{
    using namespace two_body;
    auto s = orbital_state(orbital_elements(a, M, q, e), dimensional::unit_time(t));
    double v[10] = {s.first.mass.value, s.first.position_x.value, s.first.position_y.value,
                    s.first.velocity_x.value, s.first.velocity_y.value,
                    s.second.mass.value, s.second.position_x.value, s.second.position_y.value,
                    s.second.velocity_x.value, s.second.velocity_y.value};
    std::memcpy(out, v, sizeof v);
}

// ---------------------------------------------------------------- sedov2d
// A set of T radial tracks as flat buffers: ncells[j] cells on track j,
// theta[2j], theta[2j+1] its polar bounds, radii the concatenated face radii
// (ncells[j] + 1 per track), u the concatenated conserved tuples (5 per cell:
// D, S1, S2, S3, tau, the conserved volume integrals the reference holds).
namespace {

struct FlatTracks
{
    nd::shared_array<sedov::radial_track_t, 1> tracks;
    nd::shared_array<nd::shared_array<srhd::conserved_t, 1>, 1> u;
};

FlatTracks load_tracks(int32_t T, const int64_t* ncells, const double* theta, const double* radii, const double* u)
{
    auto tr = nd::make_unique_array<sedov::radial_track_t>(nd::uivec(T));
    auto uc = nd::make_unique_array<nd::shared_array<srhd::conserved_t, 1>>(nd::uivec(T));
    for (int32_t j = 0; j < T; ++j)
    {
        auto rf = nd::make_unique_array<dimensional::unit_length>(nd::uivec(ncells[j] + 1));
        for (int64_t i = 0; i <= ncells[j]; ++i) rf(i) = *radii++;
        auto c = nd::make_unique_array<srhd::conserved_t>(nd::uivec(ncells[j]));
        for (int64_t i = 0; i < ncells[j]; ++i, u += 5) c(i) = to_tuple<srhd::conserved_t>(u);
        tr(j) = sedov::radial_track_t{nd::make_shared_array(std::move(rf)), theta[2 * j], theta[2 * j + 1]};
        uc(j) = nd::make_shared_array(std::move(c));
    }
    return {nd::make_shared_array(std::move(tr)), nd::make_shared_array(std::move(uc))};
}

// problems/sedov2d.cpp:563-587 with the boundary primitive states given per
// track (the driver takes them from its wind profile at the track's ends)
sedov::radial_godunov_data_t inner_bc(const srhd::primitive_t& ghost, const nd::shared_array<srhd::primitive_t, 1>& pc)
{
    auto vel = std::min(srhd::velocity_1(front(pc)), dimensional::unit_velocity(0.0));
    auto mode = srhd::riemann_solver_mode_hllc_fluxes_moving_face_t{vel};
    return std::pair(srhd::riemann_solver(ghost, front(pc), geometric::unit_vector_on(1), 4. / 3, mode), vel);
}

sedov::radial_godunov_data_t outer_bc(const srhd::primitive_t& ghost, const nd::shared_array<srhd::primitive_t, 1>& pc)
{
    auto vel = srhd::velocity_1(ghost);
    auto mode = srhd::riemann_solver_mode_hllc_fluxes_moving_face_t{vel};
    return std::pair(srhd::riemann_solver(back(pc), ghost, geometric::unit_vector_on(1), 4. / 3, mode), vel);
}

} // namespace

// The forward-Euler advance of problems/sedov2d.cpp:608-660 (the driver's own
// translation unit needs HDF5, so its glue is restated here around the
// reference's sedov:: scheme functions): recover_primitive, radial_gradient,
// radial_godunov_data with the inner/outer boundary Riemann data,
// polar_godunov_data between neighbouring tracks (empty track data beyond
// the poles), delta_conserved and delta_face_positions. Writes the new radii
// and conserved tuples in the input layout; optional outputs (may be null):
// prim and grad (5 per cell), radial (6 per face: flux, contact speed), and
// polar (8 per transverse face: flux, area, il, ir; for each interface
// j = 0..T-2 the ncells[j] + ncells[j+1] + 1 faces of transverse_faces).
// Returns 1 if the reference threw.
int ref_sedov_advance(int32_t T, const int64_t* ncells, const double* theta, const double* radii, const double* u,
                      const double* ghost_in, const double* ghost_out, double dt, int32_t use_plm,
                      double* radii_out, double* u_out, double* prim, double* grad, double* radial, double* polar)
{
    try
    {
        auto in = load_tracks(T, ncells, theta, radii, u);
        auto t0 = in.tracks;
        auto uc = in.u;
        std::vector<nd::shared_array<srhd::primitive_t, 1>> pc(T);
        std::vector<nd::shared_array<sedov::primitive_per_length_t, 1>> dc(T);
        std::vector<nd::shared_array<sedov::radial_godunov_data_t, 1>> ff(T);
        for (int32_t j = 0; j < T; ++j)
        {
            pc[j] = sedov::recover_primitive(t0(j), uc(j));
            dc[j] = sedov::radial_gradient(t0(j), pc[j], use_plm != 0);
            auto gi = to_tuple<srhd::primitive_t>(ghost_in + 5 * j);
            auto go = to_tuple<srhd::primitive_t>(ghost_out + 5 * j);
            ff[j] = sedov::radial_godunov_data(t0(j), pc[j], dc[j], inner_bc(gi, pc[j]), outer_bc(go, pc[j]));
        }
        auto td = [&] (int32_t j) -> sedov::track_data_t {
            if (j < 0 || j >= T) return sedov::track_data_t();
            return sedov::track_data_t{t0(j), pc[j], dc[j]};
        };
        std::vector<nd::shared_array<sedov::polar_godunov_data_t, 1>> gf(T + 1);
        for (int32_t j = 0; j + 1 < T; ++j)
            gf[j + 1] = sedov::polar_godunov_data(td(j - 1), td(j), td(j + 1), td(j + 2), use_plm != 0);
        for (int32_t j = 0; j < T; ++j)
        {
            auto du = sedov::delta_conserved(t0(j), pc[j], ff[j], gf[j], gf[j + 1], dimensional::unit_time(dt));
            auto dr = sedov::delta_face_positions(ff[j], dimensional::unit_time(dt));
            for (std::size_t i = 0; i < size(uc(j)); ++i, u_out += 5) from_tuple(uc(j)(i) + du(i), u_out);
            for (std::size_t i = 0; i < size(t0(j).face_radii); ++i) *radii_out++ = (t0(j).face_radii(i) + dr(i)).value;
            for (std::size_t i = 0; prim && i < size(pc[j]); ++i, prim += 5) from_tuple(pc[j](i), prim);
            for (std::size_t i = 0; grad && i < size(dc[j]); ++i, grad += 5) from_tuple(dc[j](i), grad);
            for (std::size_t i = 0; radial && i < size(ff[j]); ++i, radial += 6)
            {
                from_tuple(std::get<0>(ff[j](i)), radial);
                radial[5] = std::get<1>(ff[j](i)).value;
            }
        }
        for (int32_t j = 0; polar && j + 1 < T; ++j)
        {
            for (std::size_t n = 0; n < size(gf[j + 1]); ++n, polar += 8)
            {
                auto [f, da, il, ir] = gf[j + 1](n);
                from_tuple(f, polar);
                polar[5] = da.value;
                polar[6] = double(il);
                polar[7] = double(ir);
            }
        }
        return 0;
    }
    catch (const std::exception&)
    {
        return 1;
    }
}

// sedov::generate_radial_track (scheme_sedov2d.cpp:108-129): the face radii
// of a log-spaced track; returns the number of faces (written if radii is
// non-null and capacity suffices).
int64_t ref_sedov_generate_track(double r0, double r1, double theta0, double theta1, double aspect, double* radii,
                                 int64_t capacity)
{
    auto t = sedov::generate_radial_track(r0, r1, theta0, theta1, aspect);
    const int64_t n = int64_t(size(t.face_radii));
    for (int64_t i = 0; radii && i < n && i < capacity; ++i) radii[i] = t.face_radii(i).value;
    return n;
}

// sedov::remesh of one track (scheme_sedov2d.cpp:362-412): returns the new
// cell count (-1 if the reference threw); radii_out / u_out get the new
// track (capacity ncells + 1 cells).
int64_t ref_sedov_remesh(int64_t ncells, double theta0, double theta1, const double* radii, const double* u,
                         double max_aspect, double min_aspect, double inner_radius, double* radii_out, double* u_out)
{
    try
    {
        const double th[2] = {theta0, theta1};
        auto in = load_tracks(1, &ncells, th, radii, u);
        auto [t, c] = sedov::remesh(in.tracks(0), in.u(0), max_aspect, min_aspect, inner_radius);
        for (std::size_t i = 0; i < size(t.face_radii); ++i) radii_out[i] = t.face_radii(i).value;
        for (std::size_t i = 0; i < size(c); ++i) from_tuple(c(i), u_out + 5 * i);
        return int64_t(size(c));
    }
    catch (const std::exception&)
    {
        return -1;
    }
}

// sedov::cell_volume and sedov::face_area (scheme_sedov2d.cpp:40-62)
double ref_sedov_cell_volume(double r0, double r1, double t0, double t1) { return sedov::cell_volume(r0, r1, t0, t1).value; }
double ref_sedov_face_area(double r0, double r1, double t0, double t1) { return sedov::face_area(r0, r1, t0, t1).value; }

} // extern "C"
