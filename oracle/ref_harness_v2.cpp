// ORACLE — test infrastructure only (see oracle_common.hpp).
//
// C entry points around the reference's OWN mhd_scheme_v2 block API
// (src/scheme_mhd_v2.cpp:75-278), compiled by oracle/Makefile into
// oracle/_ref/libref_v2.so. The reference's scheme_mhd_v2.cpp is compiled as
// part of this translation unit: src/mesh_cartesian_3d.hpp defines
// namespace-scope lambdas without `inline`, so it can enter one translation
// unit of a library only. scheme_mhd_v2 also needs the bsp::tree_index_t
// alias of ref_v2_alias.hpp, which the Makefile force-includes. Block arrays
// go in and out as flat AoS tuples (conserved 5, primitive 8, godunov data 8)
// or scalars (face fields, edge EMFs); every entry returns 1 if the reference
// threw.
#include <array>
#include <cstdint>
#include "scheme_mhd_v2.cpp"
#include "ref_marshal.hpp"

namespace {

using v2_face_b = mhd_scheme_v2::face_magnetic_flux_density_t;
using v2_edge_e = mhd_scheme_v2::edge_electromotive_density_t;
using v2_face_g = mhd_scheme_v2::face_godunov_data_t;

v2_face_b v2_faces(const double* const b[3], const std::array<nd::uivec_t<3>, 3>& sh)
{
    return {make_scalar3<mhd::unit_magnetic_field>(b[0], sh[0][0], sh[0][1], sh[0][2]),
            make_scalar3<mhd::unit_magnetic_field>(b[1], sh[1][0], sh[1][1], sh[1][2]),
            make_scalar3<mhd::unit_magnetic_field>(b[2], sh[2][0], sh[2][1], sh[2][2])};
}

v2_edge_e v2_edges(const double* const e[3], const std::array<nd::uivec_t<3>, 3>& sh)
{
    return {make_scalar3<mhd::unit_electric_field>(e[0], sh[0][0], sh[0][1], sh[0][2]),
            make_scalar3<mhd::unit_electric_field>(e[1], sh[1][0], sh[1][1], sh[1][2]),
            make_scalar3<mhd::unit_electric_field>(e[2], sh[2][0], sh[2][1], sh[2][2])};
}

v2_face_g v2_godunov(const double* const g[3], const std::array<nd::uivec_t<3>, 3>& sh)
{
    return {make_array3<mhd::godunov_data_t>(g[0], sh[0][0], sh[0][1], sh[0][2]),
            make_array3<mhd::godunov_data_t>(g[1], sh[1][0], sh[1][1], sh[1][2]),
            make_array3<mhd::godunov_data_t>(g[2], sh[2][0], sh[2][1], sh[2][2])};
}

} // namespace

extern "C" {

// primitive_array: uc (n0, n1, n2) cells, bf faces (+1 along their axis)
int ref_mhd_v2_primitive_array(int32_t n0, int32_t n1, int32_t n2, const double* uc, const double* bf1,
                               const double* bf2, const double* bf3, double* pc)
{
    try {
        const double* b[3] = {bf1, bf2, bf3};
        auto u = make_array3<mhd::conserved_density_t>(uc, n0, n1, n2);
        read_array3(mhd_scheme_v2::primitive_array(u, v2_faces(b, staggered_shapes(n0, n1, n2, 1, 0))), pc);
        return 0;
    } catch (...) {
        return 1;
    }
}

// godunov_fluxes: pc (m0, m1, m2) cells, bf faces (-1 along their axis);
// gf (-1 along their axis) godunov 8-tuples
int ref_mhd_v2_godunov_fluxes(int32_t m0, int32_t m1, int32_t m2, const double* pc, const double* bf1,
                              const double* bf2, const double* bf3, double* gf1, double* gf2, double* gf3)
{
    try {
        const double* b[3] = {bf1, bf2, bf3};
        auto p = make_array3<mhd::primitive_t>(pc, m0, m1, m2);
        auto g = mhd_scheme_v2::godunov_fluxes(p, v2_faces(b, staggered_shapes(m0, m1, m2, -1, 0)));
        read_array3(g[0], gf1);
        read_array3(g[1], gf2);
        read_array3(g[2], gf3);
        return 0;
    } catch (...) {
        return 1;
    }
}

// electromotive_forces: gf of a (m0, m1, m2) cell array (-1 along their
// axis); ee (-1 on the two axes other than their own)
int ref_mhd_v2_electromotive_forces(int32_t m0, int32_t m1, int32_t m2, const double* gf1, const double* gf2,
                                    const double* gf3, double* ee1, double* ee2, double* ee3)
{
    try {
        const double* g[3] = {gf1, gf2, gf3};
        auto e = mhd_scheme_v2::electromotive_forces(v2_godunov(g, staggered_shapes(m0, m1, m2, -1, 0)));
        read_scalar3(e[0], ee1);
        read_scalar3(e[1], ee2);
        read_scalar3(e[2], ee3);
        return 0;
    } catch (...) {
        return 1;
    }
}

// updated_conserved_density: uc (n0, n1, n2); gf (+1 along their axis, +2
// on the others)
int ref_mhd_v2_updated_conserved_density(int32_t n0, int32_t n1, int32_t n2, const double* uc, const double* gf1,
                                         const double* gf2, const double* gf3, double dt, double dl, double* out)
{
    try {
        const double* g[3] = {gf1, gf2, gf3};
        auto u = make_array3<mhd::conserved_density_t>(uc, n0, n1, n2);
        read_array3(mhd_scheme_v2::updated_conserved_density(u, v2_godunov(g, staggered_shapes(n0, n1, n2, 1, 2)),
                                                             dimensional::unit_time(dt),
                                                             dimensional::unit_length(dl)), out);
        return 0;
    } catch (...) {
        return 1;
    }
}

// curl: edges of a (n0, n1, n2) block (+1 on the two axes other than their
// own); cf faces (+1 along their axis)
int ref_mhd_v2_curl(int32_t n0, int32_t n1, int32_t n2, const double* ee1, const double* ee2, const double* ee3,
                    double dl, double* cf1, double* cf2, double* cf3)
{
    try {
        const double* e[3] = {ee1, ee2, ee3};
        auto sh = staggered_shapes(n0, n1, n2, 0, 1);
        auto c = mhd_scheme_v2::curl(v2_edges(e, sh), dimensional::unit_length(dl));
        read_scalar3(c[0], cf1);
        read_scalar3(c[1], cf2);
        read_scalar3(c[2], cf3);
        return 0;
    } catch (...) {
        return 1;
    }
}

// updated_magnetic_flux_density: bf faces of a (n0, n1, n2) block (+1 along
// their axis); ee edges as electromotive_forces gives them for the block
// extended by one cell on every side (+2 along their axis, +1 on the others)
int ref_mhd_v2_updated_magnetic_flux_density(int32_t n0, int32_t n1, int32_t n2, const double* bf1,
                                             const double* bf2, const double* bf3, const double* ee1,
                                             const double* ee2, const double* ee3, double dt, double dl,
                                             double* out1, double* out2, double* out3)
{
    try {
        const double* b[3] = {bf1, bf2, bf3};
        const double* e[3] = {ee1, ee2, ee3};
        auto r = mhd_scheme_v2::updated_magnetic_flux_density(
            v2_faces(b, staggered_shapes(n0, n1, n2, 1, 0)), v2_edges(e, staggered_shapes(n0, n1, n2, 2, 1)),
            dimensional::unit_time(dt), dimensional::unit_length(dl));
        read_scalar3(r[0], out1);
        read_scalar3(r[1], out2);
        read_scalar3(r[2], out3);
        return 0;
    } catch (...) {
        return 1;
    }
}

} // extern "C"
