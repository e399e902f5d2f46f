// The reference's split, per-block MHD API and its pointwise physics, FP64 on
// the GPU:
//   mhd_scheme_v2::primitive_array, godunov_fluxes, electromotive_forces,
//   updated_conserved_density, curl, updated_magnetic_flux_density
//   (src/scheme_mhd_v2.cpp:75-278), on block arrays in the reference's AoS
//   tuple layout (conserved 5, primitive 8, godunov data 8 = flux 5 + E 3;
//   face fields and edge EMFs as scalars), row-major, last axis contiguous;
//   mhd::recover_primitive, conserved_density, flux, fast_speed_squared,
//   fastest_speed, riemann_hlle (src/physics_mhd.hpp:216-390) and
//   iso2d::flux, outer_wavespeeds, fastest_wavespeed, riemann_hlle
//   (src/physics_iso2d.hpp:99-173) on batches of points.
// One thread per output element; every kernel is a gather of its stencil
// from global memory (these calls move a block per call, the whole-cube
// path of mhd.cu is the fast one). Arithmetic follows the reference's
// evaluation order; FMA contraction is the only difference.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include "common.cuh"
#include "mhd_physics.cuh"

namespace mara {
namespace mhdv2 {

using mhd::Prim;

struct Shape
{
    int n0, n1, n2;
    __host__ __device__ int64_t size() const { return int64_t(n0) * n1 * n2; }
    __host__ __device__ int64_t at(int i, int j, int k) const { return (int64_t(i) * n1 + j) * n2 + k; }
    __device__ void split(int64_t t, int& i, int& j, int& k) const
    {
        k = int(t % n2);
        t /= n2;
        j = int(t % n1);
        i = int(t / n1);
    }
};

// the array of `axis` (0..2) of a staggered triple: `grow` added along its own
// axis, `side` along the two others
__host__ __device__ inline Shape staggered(Shape c, int axis, int grow, int side)
{
    return Shape{c.n0 + (axis == 0 ? grow : side), c.n1 + (axis == 1 ? grow : side), c.n2 + (axis == 2 ? grow : side)};
}

__device__ inline int64_t step(const Shape& s, int axis) { return axis == 0 ? int64_t(s.n1) * s.n2 : (axis == 1 ? s.n2 : 1); }

__device__ inline Prim<double> load_prim(const double* p)
{
    Prim<double> q;
    q.d = p[0];
    for (int k = 0; k < 3; ++k) q.v[k] = p[1 + k];
    q.p = p[4];
    for (int k = 0; k < 3; ++k) q.b[k] = p[5 + k];
    return q;
}

__device__ inline void store_prim(double* out, const Prim<double>& p)
{
    out[0] = p.d;
    for (int k = 0; k < 3; ++k) out[1 + k] = p.v[k];
    out[4] = p.p;
    for (int k = 0; k < 3; ++k) out[5 + k] = p.b[k];
}

#define MARA_GRID_LOOP(t, n) for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < (n); t += int64_t(gridDim.x) * blockDim.x)

// primitive_array (scheme_mhd_v2.cpp:75-81): face_to_cell by adjacent means,
// then recover_primitive
__global__ void primitive_kernel(Shape c, const double* uc, const double* bf1, const double* bf2, const double* bf3,
                                 double gamma, double* pc, unsigned long long* failures)
{
    const Shape f0 = staggered(c, 0, 1, 0), f1 = staggered(c, 1, 1, 0), f2 = staggered(c, 2, 1, 0);
    unsigned long long bad = 0;
    MARA_GRID_LOOP(t, c.size())
    {
        int i, j, k;
        c.split(t, i, j, k);
        const double b[3] = {0.5 * (bf1[f0.at(i, j, k)] + bf1[f0.at(i + 1, j, k)]),
                             0.5 * (bf2[f1.at(i, j, k)] + bf2[f1.at(i, j + 1, k)]),
                             0.5 * (bf3[f2.at(i, j, k)] + bf3[f2.at(i, j, k + 1)])};
        Prim<double> p;
        bad += mhd::recover_primitive(uc + 5 * t, b, gamma, p) ? 0 : 1;
        store_prim(pc + 8 * t, p);
    }
    if (failures && bad) atomicAdd(failures, bad);
}

// godunov_fluxes (scheme_mhd_v2.cpp:143-163) across the faces of `AXIS`
// between the cells of pc (shape m); godunov data = HLLE flux, then the
// E-field with its normal component zero
template<int AXIS>
__global__ void godunov_kernel(Shape m, const double* pc, const double* bf, double gamma, double* gf)
{
    const Shape f = staggered(m, AXIS, -1, 0);
    const int64_t d = step(m, AXIS);
    MARA_GRID_LOOP(t, f.size())
    {
        int i, j, k;
        f.split(t, i, j, k);
        const int64_t c = m.at(i, j, k);
        double F[5], Et[2];
        mhd::riemann_hlle<double, AXIS>(load_prim(pc + 8 * c), load_prim(pc + 8 * (c + d)), bf[t], gamma, F, Et);
        double* g = gf + 8 * t;
        for (int q = 0; q < 5; ++q) g[q] = F[q];
        g[5 + AXIS] = 0.0;
        g[5 + (AXIS == 0 ? 1 : 0)] = Et[0];
        g[5 + (AXIS == 2 ? 1 : 2)] = Et[1];
    }
}

// electromotive_forces (scheme_mhd_v2.cpp:168-192): the edge EMF of axis a
// is the mean of the two adjacent means of E_a over the faces of the two
// other axes, the ee1 = 0.5 * (gf2|a3 + gf3|a2) pattern
__global__ void emf_kernel(Shape m, const double* gf1, const double* gf2, const double* gf3, double* ee1, double* ee2,
                           double* ee3)
{
    const Shape g0 = staggered(m, 0, -1, 0), g1 = staggered(m, 1, -1, 0), g2 = staggered(m, 2, -1, 0);
    const Shape e0 = staggered(m, 0, 0, -1), e1 = staggered(m, 1, 0, -1), e2 = staggered(m, 2, 0, -1);
    const int64_t n0 = e0.size(), n1 = e1.size();
    MARA_GRID_LOOP(t, n0 + n1 + e2.size())
    {
        int i, j, k;
        if (t < n0)
        {
            e0.split(t, i, j, k);
            const double a = 0.5 * (gf2[8 * g1.at(i, j, k) + 5] + gf2[8 * g1.at(i, j, k + 1) + 5]);
            const double b = 0.5 * (gf3[8 * g2.at(i, j, k) + 5] + gf3[8 * g2.at(i, j + 1, k) + 5]);
            ee1[t] = 0.5 * (a + b);
        }
        else if (t < n0 + n1)
        {
            const int64_t u = t - n0;
            e1.split(u, i, j, k);
            const double a = 0.5 * (gf3[8 * g2.at(i, j, k) + 6] + gf3[8 * g2.at(i + 1, j, k) + 6]);
            const double b = 0.5 * (gf1[8 * g0.at(i, j, k) + 6] + gf1[8 * g0.at(i, j, k + 1) + 6]);
            ee2[u] = 0.5 * (a + b);
        }
        else
        {
            const int64_t u = t - n0 - n1;
            e2.split(u, i, j, k);
            const double a = 0.5 * (gf1[8 * g0.at(i, j, k) + 7] + gf1[8 * g0.at(i, j + 1, k) + 7]);
            const double b = 0.5 * (gf2[8 * g1.at(i, j, k) + 7] + gf2[8 * g1.at(i + 1, j, k) + 7]);
            ee3[u] = 0.5 * (a + b);
        }
    }
}

// updated_conserved_density (scheme_mhd_v2.cpp:197-219): the godunov fluxes
// come extended by one zone on the transverse axes (remove_transverse(1)
// picks the block's own faces), uc - div F dt / dl
__global__ void update_conserved_kernel(Shape c, const double* uc, const double* gf1, const double* gf2,
                                        const double* gf3, double dt, double dl, double* out)
{
    const Shape g0 = staggered(c, 0, 1, 2), g1 = staggered(c, 1, 1, 2), g2 = staggered(c, 2, 1, 2);
    MARA_GRID_LOOP(t, c.size())
    {
        int i, j, k;
        c.split(t, i, j, k);
        const double* a0 = gf1 + 8 * g0.at(i, j + 1, k + 1);
        const double* a1 = gf1 + 8 * g0.at(i + 1, j + 1, k + 1);
        const double* b0 = gf2 + 8 * g1.at(i + 1, j, k + 1);
        const double* b1 = gf2 + 8 * g1.at(i + 1, j + 1, k + 1);
        const double* c0 = gf3 + 8 * g2.at(i + 1, j + 1, k);
        const double* c1 = gf3 + 8 * g2.at(i + 1, j + 1, k + 1);
        for (int q = 0; q < 5; ++q)
        {
            const double div = ((a1[q] - a0[q]) + (b1[q] - b0[q])) + (c1[q] - c0[q]);
            out[5 * t + q] = uc[5 * t + q] - div * dt / dl;
        }
    }
}

// solenoidal_difference (src/mesh_cartesian_3d.hpp:266-273) of edge arrays
// e1 [n0][n1+1][n2+1], e2 [n0+1][n1][n2+1], e3 [n0+1][n1+1][n2] reached
// through offsets o (rl: the longitudinal layer removed, as
// updated_magnetic_flux_density does) into arrays of shapes s; out_k =
// base_k - cf_k * dt / dl, or cf_k * dt / dl where base is null (curl)
__global__ void solenoidal_kernel(Shape c, const double* e1, const double* e2, const double* e3, Shape s1, Shape s2,
                                  Shape s3, int rl, const double* b1, const double* b2, const double* b3, double dt,
                                  double dl, double* o1, double* o2, double* o3)
{
    const Shape f0 = staggered(c, 0, 1, 0), f1 = staggered(c, 1, 1, 0), f2 = staggered(c, 2, 1, 0);
    const int64_t n0 = f0.size(), n1 = f1.size();
    // the edges of the block's own faces: e1(i, j, k) = ee1(i + rl, j, k) etc.
    auto E1 = [&] (int i, int j, int k) { return e1[s1.at(i + rl, j, k)]; };
    auto E2 = [&] (int i, int j, int k) { return e2[s2.at(i, j + rl, k)]; };
    auto E3 = [&] (int i, int j, int k) { return e3[s3.at(i, j, k + rl)]; };
    MARA_GRID_LOOP(t, n0 + n1 + f2.size())
    {
        int i, j, k;
        double cf;
        const double* base;
        double* out;
        int64_t u;
        if (t < n0)
        {
            u = t;
            f0.split(u, i, j, k);
            cf = (E3(i, j + 1, k) - E3(i, j, k)) - (E2(i, j, k + 1) - E2(i, j, k));
            base = b1;
            out = o1;
        }
        else if (t < n0 + n1)
        {
            u = t - n0;
            f1.split(u, i, j, k);
            cf = (E1(i, j, k + 1) - E1(i, j, k)) - (E3(i + 1, j, k) - E3(i, j, k));
            base = b2;
            out = o2;
        }
        else
        {
            u = t - n0 - n1;
            f2.split(u, i, j, k);
            cf = (E2(i + 1, j, k) - E2(i, j, k)) - (E1(i, j + 1, k) - E1(i, j, k));
            base = b3;
            out = o3;
        }
        out[u] = base ? base[u] - cf * dt / dl : cf * dt / dl;
    }
}

// ---- pointwise physics on batches
template<int AXIS>
__device__ inline void flux_at(const Prim<double>& p, double gm, double f[5])
{
    // mhd::flux (physics_mhd.hpp:324-349): vn u + pressure term + Maxwell term
    double u[5];
    mhd::conserved(p, gm, u);
    const double bn = p.b[AXIS], vn = p.v[AXIS];
    const double pt = p.p + 0.5 * mhd::sum3(p.b, p.b);
    const double bv = mhd::sum3(p.b, p.v);
    f[0] = vn * u[0];
    for (int k = 0; k < 3; ++k) f[1 + k] = vn * u[1 + k] + (k == AXIS ? pt : 0.0) + -bn * p.b[k];
    f[4] = vn * u[4] + pt * vn + -bn * bv;
}

template<int AXIS>
__device__ inline double fast_speed_squared_at(const Prim<double>& p, double gm)
{
    // mhd::fast_speed_squared (physics_mhd.hpp:216-222)
    const double cs2 = gm * p.p / p.d;
    const double va2 = mhd::sum3(p.b, p.b) / p.d;
    const double van2 = (p.b[AXIS] * p.b[AXIS]) / p.d;
    const double cf2 = cs2 + va2;
    const double cg2 = sqrt(cf2 * cf2 - 4.0 * cs2 * van2);
    return 0.5 * (cf2 + cg2);
}

template<int AXIS>
__global__ void mhd_point_kernel(const double* p, const double* pr, const double* bl, int64_t n, double gm, int what,
                                 double* out)
{
    MARA_GRID_LOOP(t, n)
    {
        const Prim<double> a = load_prim(p + 8 * t);
        if (what == 0) flux_at<AXIS>(a, gm, out + 5 * t);
        else if (what == 1) out[t] = fast_speed_squared_at<AXIS>(a, gm);
        else if (what == 2) out[t] = mhd::fastest_speed(a, gm);
        else if (what == 3) mhd::conserved(a, gm, out + 5 * t);
        else
        {
            double F[5], Et[2];
            mhd::riemann_hlle<double, AXIS>(a, load_prim(pr + 8 * t), bl[t], gm, F, Et);
            double* g = out + 8 * t;
            for (int q = 0; q < 5; ++q) g[q] = F[q];
            g[5 + AXIS] = 0.0;
            g[5 + (AXIS == 0 ? 1 : 0)] = Et[0];
            g[5 + (AXIS == 2 ? 1 : 2)] = Et[1];
        }
    }
}

__global__ void mhd_recover_kernel(const double* u, const double* b, int64_t n, double gm, double* p, int32_t* status,
                                   unsigned long long* failures)
{
    unsigned long long bad = 0;
    MARA_GRID_LOOP(t, n)
    {
        Prim<double> q;
        const bool ok = mhd::recover_primitive(u + 5 * t, b + 3 * t, gm, q);
        store_prim(p + 8 * t, q);
        if (status) status[t] = ok ? 0 : 1;
        bad += ok ? 0 : 1;
    }
    if (failures && bad) atomicAdd(failures, bad);
}

// iso2d (physics_iso2d.hpp:99-173) at axis-aligned normals: p = (Sigma, v1, v2)
template<int AXIS>
__device__ inline void iso2d_flux(const double p[3], double cs2, double f[3])
{
    const double pg = p[0] * cs2;
    const double vn = p[1 + AXIS];
    const double u[3] = {p[0], p[0] * p[1], p[0] * p[2]};
    f[0] = vn * u[0] + 0.0;
    f[1] = vn * u[1] + (AXIS == 0 ? pg : 0.0);
    f[2] = vn * u[2] + (AXIS == 1 ? pg : 0.0);
}

template<int AXIS>
__device__ inline void iso2d_outer(const double p[3], double cs2, double& am, double& ap)
{
    const double vn = p[1 + AXIS];
    const double cs = sqrt(cs2);
    am = vn - cs;
    ap = vn + cs;
}

template<int AXIS>
__global__ void iso2d_point_kernel(const double* pl, const double* pr, const double* cs2v, int64_t n, int what,
                                   double* out)
{
    MARA_GRID_LOOP(t, n)
    {
        const double* a = pl + 3 * t;
        const double cs2 = cs2v[t];
        if (what == 0) iso2d_flux<AXIS>(a, cs2, out + 3 * t);
        else if (what == 1) iso2d_outer<AXIS>(a, cs2, out[2 * t], out[2 * t + 1]);
        else if (what == 2)
        {
            double m0, p0, m1, p1;
            iso2d_outer<0>(a, cs2, m0, p0);
            iso2d_outer<1>(a, cs2, m1, p1);
            out[t] = fmax(fmax(fabs(m0), fabs(p0)), fmax(fabs(m1), fabs(p1)));
        }
        else
        {
            // riemann_hlle (physics_iso2d.hpp:156-173)
            const double* b = pr + 3 * t;
            const double ul[3] = {a[0], a[0] * a[1], a[0] * a[2]};
            const double ur[3] = {b[0], b[0] * b[1], b[0] * b[2]};
            double fl[3], fr[3], alm, alp, arm, arp;
            iso2d_flux<AXIS>(a, cs2, fl);
            iso2d_flux<AXIS>(b, cs2, fr);
            iso2d_outer<AXIS>(a, cs2, alm, alp);
            iso2d_outer<AXIS>(b, cs2, arm, arp);
            const double ap = fmax(0.0, fmax(alp, arp));
            const double am = fmin(0.0, fmin(alm, arm));
            for (int k = 0; k < 3; ++k)
                out[3 * t + k] = (ap * fl[k] - am * fr[k] - (ul[k] - ur[k]) * ap * am) / (ap - am);
        }
    }
}

#undef MARA_GRID_LOOP

inline int blocks(int64_t n) { return int(std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 8))); }

inline bool positive(int a, int b, int c) { return a > 0 && b > 0 && c > 0; }

template<typename K, typename... Args>
int launch(const char* what, int64_t n, cudaStream_t s, K kernel, Args... args)
{
    if (n <= 0) return MARA_OK;
    kernel<<<blocks(n), 256, 0, s>>>(args...);
    return launch_status(what);
}

} // namespace mhdv2
} // namespace mara

using mara::mhdv2::Shape;
using mara::mhdv2::staggered;

extern "C" {

int mara_mhd_v2_primitive_array(int32_t n0, int32_t n1, int32_t n2, const double* uc, const double* bf1,
                                const double* bf2, const double* bf3, double gamma_law_index, double* pc,
                                unsigned long long* failures, void* stream)
{
    MARA_REQUIRE(mara::mhdv2::positive(n0, n1, n2), "mara_mhd_v2_primitive_array: block shape must be positive");
    MARA_REQUIRE(uc && bf1 && bf2 && bf3 && pc, "mara_mhd_v2_primitive_array: null buffer");
    const Shape c{n0, n1, n2};
    return mara::mhdv2::launch("mhd v2 primitive_kernel", c.size(), mara::as_stream(stream),
                               mara::mhdv2::primitive_kernel, c, uc, bf1, bf2, bf3, gamma_law_index, pc, failures);
}

int mara_mhd_v2_godunov_fluxes(int32_t m0, int32_t m1, int32_t m2, const double* pc, const double* bf1,
                               const double* bf2, const double* bf3, double gamma_law_index, double* gf1,
                               double* gf2, double* gf3, void* stream)
{
    MARA_REQUIRE(m0 > 1 && m1 > 1 && m2 > 1, "mara_mhd_v2_godunov_fluxes: the cell array needs two cells per axis");
    MARA_REQUIRE(pc && bf1 && bf2 && bf3 && gf1 && gf2 && gf3, "mara_mhd_v2_godunov_fluxes: null buffer");
    const Shape m{m0, m1, m2};
    cudaStream_t s = mara::as_stream(stream);
    using namespace mara::mhdv2;
    if (int r = launch("mhd v2 godunov_kernel<0>", staggered(m, 0, -1, 0).size(), s, godunov_kernel<0>, m, pc, bf1,
                       gamma_law_index, gf1))
        return r;
    if (int r = launch("mhd v2 godunov_kernel<1>", staggered(m, 1, -1, 0).size(), s, godunov_kernel<1>, m, pc, bf2,
                       gamma_law_index, gf2))
        return r;
    return launch("mhd v2 godunov_kernel<2>", staggered(m, 2, -1, 0).size(), s, godunov_kernel<2>, m, pc, bf3,
                  gamma_law_index, gf3);
}

int mara_mhd_v2_electromotive_forces(int32_t m0, int32_t m1, int32_t m2, const double* gf1, const double* gf2,
                                     const double* gf3, double* ee1, double* ee2, double* ee3, void* stream)
{
    MARA_REQUIRE(m0 > 1 && m1 > 1 && m2 > 1,
                 "mara_mhd_v2_electromotive_forces: the cell array needs two cells per axis");
    MARA_REQUIRE(gf1 && gf2 && gf3 && ee1 && ee2 && ee3, "mara_mhd_v2_electromotive_forces: null buffer");
    const Shape m{m0, m1, m2};
    const int64_t n = staggered(m, 0, 0, -1).size() + staggered(m, 1, 0, -1).size() + staggered(m, 2, 0, -1).size();
    return mara::mhdv2::launch("mhd v2 emf_kernel", n, mara::as_stream(stream), mara::mhdv2::emf_kernel, m, gf1, gf2,
                               gf3, ee1, ee2, ee3);
}

int mara_mhd_v2_updated_conserved_density(int32_t n0, int32_t n1, int32_t n2, const double* uc, const double* gf1,
                                          const double* gf2, const double* gf3, double dt, double dl,
                                          double* uc_out, void* stream)
{
    MARA_REQUIRE(mara::mhdv2::positive(n0, n1, n2), "mara_mhd_v2_updated_conserved_density: block shape must be positive");
    MARA_REQUIRE(uc && gf1 && gf2 && gf3 && uc_out, "mara_mhd_v2_updated_conserved_density: null buffer");
    MARA_REQUIRE(dl > 0.0, "mara_mhd_v2_updated_conserved_density: dl must be positive");
    const Shape c{n0, n1, n2};
    return mara::mhdv2::launch("mhd v2 update_conserved_kernel", c.size(), mara::as_stream(stream),
                               mara::mhdv2::update_conserved_kernel, c, uc, gf1, gf2, gf3, dt, dl, uc_out);
}

int mara_mhd_v2_curl(int32_t n0, int32_t n1, int32_t n2, const double* ee1, const double* ee2, const double* ee3,
                     double dl, double* cf1, double* cf2, double* cf3, void* stream)
{
    MARA_REQUIRE(mara::mhdv2::positive(n0, n1, n2), "mara_mhd_v2_curl: block shape must be positive");
    MARA_REQUIRE(ee1 && ee2 && ee3 && cf1 && cf2 && cf3, "mara_mhd_v2_curl: null buffer");
    MARA_REQUIRE(dl > 0.0, "mara_mhd_v2_curl: dl must be positive");
    const Shape c{n0, n1, n2};
    const int64_t n = staggered(c, 0, 1, 0).size() + staggered(c, 1, 1, 0).size() + staggered(c, 2, 1, 0).size();
    return mara::mhdv2::launch("mhd v2 solenoidal_kernel (curl)", n, mara::as_stream(stream),
                               mara::mhdv2::solenoidal_kernel, c, ee1, ee2, ee3, staggered(c, 0, 0, 1),
                               staggered(c, 1, 0, 1), staggered(c, 2, 0, 1), 0, (const double*)nullptr,
                               (const double*)nullptr, (const double*)nullptr, 1.0, dl, cf1, cf2, cf3);
}

int mara_mhd_v2_updated_magnetic_flux_density(int32_t n0, int32_t n1, int32_t n2, const double* bf1,
                                              const double* bf2, const double* bf3, const double* ee1,
                                              const double* ee2, const double* ee3, double dt, double dl,
                                              double* bf1_out, double* bf2_out, double* bf3_out, void* stream)
{
    MARA_REQUIRE(mara::mhdv2::positive(n0, n1, n2),
                 "mara_mhd_v2_updated_magnetic_flux_density: block shape must be positive");
    MARA_REQUIRE(bf1 && bf2 && bf3 && ee1 && ee2 && ee3 && bf1_out && bf2_out && bf3_out,
                 "mara_mhd_v2_updated_magnetic_flux_density: null buffer");
    MARA_REQUIRE(dl > 0.0, "mara_mhd_v2_updated_magnetic_flux_density: dl must be positive");
    const Shape c{n0, n1, n2};
    const int64_t n = staggered(c, 0, 1, 0).size() + staggered(c, 1, 1, 0).size() + staggered(c, 2, 1, 0).size();
    return mara::mhdv2::launch("mhd v2 solenoidal_kernel (update)", n, mara::as_stream(stream),
                               mara::mhdv2::solenoidal_kernel, c, ee1, ee2, ee3, staggered(c, 0, 2, 1),
                               staggered(c, 1, 2, 1), staggered(c, 2, 2, 1), 1, bf1, bf2, bf3, dt, dl, bf1_out,
                               bf2_out, bf3_out);
}

int mara_mhd_recover_primitive(const double* u, const double* b, int64_t n, double gamma_law_index, double* p,
                               int32_t* status, unsigned long long* failures, void* stream)
{
    MARA_REQUIRE(n >= 0, "mara_mhd_recover_primitive: negative count");
    MARA_REQUIRE(n == 0 || (u && b && p), "mara_mhd_recover_primitive: null buffer");
    return mara::mhdv2::launch("mhd_recover_kernel", n, mara::as_stream(stream), mara::mhdv2::mhd_recover_kernel, u,
                               b, n, gamma_law_index, p, status, failures);
}

namespace {

int mhd_point(const char* name, const double* p, const double* pr, const double* bl, int64_t n, int32_t axis,
              double gm, int what, double* out, void* stream)
{
    using namespace mara::mhdv2;
    MARA_REQUIRE(n >= 0, std::string(name) + ": negative count");
    MARA_REQUIRE(n == 0 || (p && out), std::string(name) + ": null buffer");
    MARA_REQUIRE(axis >= 1 && axis <= 3, std::string(name) + ": axis must be 1, 2 or 3");
    cudaStream_t s = mara::as_stream(stream);
    if (axis == 1) return launch(name, n, s, mhd_point_kernel<0>, p, pr, bl, n, gm, what, out);
    if (axis == 2) return launch(name, n, s, mhd_point_kernel<1>, p, pr, bl, n, gm, what, out);
    return launch(name, n, s, mhd_point_kernel<2>, p, pr, bl, n, gm, what, out);
}

int iso2d_point(const char* name, const double* pl, const double* pr, const double* cs2, int64_t n, int32_t axis,
                int what, double* out, void* stream)
{
    using namespace mara::mhdv2;
    MARA_REQUIRE(n >= 0, std::string(name) + ": negative count");
    MARA_REQUIRE(n == 0 || (pl && cs2 && out), std::string(name) + ": null buffer");
    MARA_REQUIRE(axis == 1 || axis == 2, std::string(name) + ": axis must be 1 or 2");
    cudaStream_t s = mara::as_stream(stream);
    if (axis == 1) return launch(name, n, s, iso2d_point_kernel<0>, pl, pr, cs2, n, what, out);
    return launch(name, n, s, iso2d_point_kernel<1>, pl, pr, cs2, n, what, out);
}

} // namespace

int mara_mhd_conserved_density(const double* p, int64_t n, double gamma_law_index, double* u, void* stream)
{
    return mhd_point("mara_mhd_conserved_density", p, nullptr, nullptr, n, 1, gamma_law_index, 3, u, stream);
}

int mara_mhd_flux(const double* p, int64_t n, int32_t axis, double gamma_law_index, double* f, void* stream)
{
    return mhd_point("mara_mhd_flux", p, nullptr, nullptr, n, axis, gamma_law_index, 0, f, stream);
}

int mara_mhd_fast_speed_squared(const double* p, int64_t n, int32_t axis, double gamma_law_index, double* out,
                                void* stream)
{
    return mhd_point("mara_mhd_fast_speed_squared", p, nullptr, nullptr, n, axis, gamma_law_index, 1, out, stream);
}

int mara_mhd_fastest_speed(const double* p, int64_t n, double gamma_law_index, double* out, void* stream)
{
    return mhd_point("mara_mhd_fastest_speed", p, nullptr, nullptr, n, 1, gamma_law_index, 2, out, stream);
}

int mara_mhd_riemann_hlle(const double* pl, const double* pr, const double* b_longitudinal, int64_t n, int32_t axis,
                          double gamma_law_index, double* out, void* stream)
{
    MARA_REQUIRE(n == 0 || (pr && b_longitudinal), "mara_mhd_riemann_hlle: null buffer");
    return mhd_point("mara_mhd_riemann_hlle", pl, pr, b_longitudinal, n, axis, gamma_law_index, 4, out, stream);
}

int mara_iso2d_flux(const double* p, const double* cs2, int64_t n, int32_t axis, double* f, void* stream)
{
    return iso2d_point("mara_iso2d_flux", p, nullptr, cs2, n, axis, 0, f, stream);
}

int mara_iso2d_outer_wavespeeds(const double* p, const double* cs2, int64_t n, int32_t axis, double* out,
                                void* stream)
{
    return iso2d_point("mara_iso2d_outer_wavespeeds", p, nullptr, cs2, n, axis, 1, out, stream);
}

int mara_iso2d_fastest_wavespeed(const double* p, const double* cs2, int64_t n, double* out, void* stream)
{
    return iso2d_point("mara_iso2d_fastest_wavespeed", p, nullptr, cs2, n, 1, 2, out, stream);
}

int mara_iso2d_riemann_hlle(const double* pl, const double* pr, const double* cs2, int64_t n, int32_t axis,
                            double* f, void* stream)
{
    MARA_REQUIRE(n == 0 || pr, "mara_iso2d_riemann_hlle: null buffer");
    return iso2d_point("mara_iso2d_riemann_hlle", pl, pr, cs2, n, axis, 3, f, stream);
}

} // extern "C"
