// Spherical-track SRHD (the sedov2d scheme) on the GPU: the per-stage
// functions of src/scheme_sedov2d.cpp:150-356 over a set of radial tracks,
// with the boundary Riemann data of problems/sedov2d.cpp:563-587 and the RK
// combinations of src/app_control.hpp:169-195 (weighted_sum of radii and
// conserved, problems/sedov2d.cpp:127-152). gamma = 4/3, temperature floor 1e-6.
//
// Layout (device): T tracks in CSR form. cell_offset[T+1] (int64) gives the
// first cell of each track; track j has n_j = cell_offset[j+1] - cell_offset[j]
// cells and n_j + 1 face radii starting at radii[cell_offset[j] + j];
// theta[2j], theta[2j+1] bound it in the polar angle. Conserved volume
// integrals are SoA u[5][C] (D, S1, S2, S3, tau). The transverse (polar)
// faces of the interface between tracks j and j+1 are the n_j + n_{j+1} + 1
// adjacent pairs of the merged face radii of both tracks
// (mesh::transverse_faces, src/mesh_sliding.hpp:122-172); interface j's
// faces start at po(j) = co[j] + co[j+1] - co[1] + j.
//
// Each call first tabulates the tracks' sines, cosines and centre cotangents
// (trig_kernel); then one stage = five kernels, one thread per item:
//   prim_kernel    cell: volume, u / dV, SRHD Newton recovery
//   grad_kernel    cell: PLM slope on the cell-centre radii (zero at both ends)
//   radial_kernel  face: faces states from both neighbours' slopes, HLLC flux
//                  across the contact and the contact speed;
//                  boundary faces: moving-face HLLC against the ghost states;
//                  moves the face by speed * dt (and the RK combination)
//   polar_kernel   transverse face: merge-path position in the two tracks'
//                  radii, samples, PLM in theta, fixed-face HLLC, face area
//   update_kernel  cell: radial flux differences, the polar fluxes binned on
//                  the cell in face order, spherical source terms, u + du
//                  (and the RK combination)
// The slopes are stored once per cell: every radial face reads two and every
// transverse face samples up to four (each slope costs 15 FP64 divisions,
// and FP64 runs at a small fraction of the FP32 rate on this part).
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdint>
#include "common.cuh"
#include "srhd_physics.cuh"

namespace mara {
namespace sedov {

using srhd::SPrim;

constexpr double kGamma = 4. / 3;
constexpr double kFloor = 1e-6;

struct Tracks
{
    int T;
    int64_t C;
    const int64_t* co;
    const double* theta;
};

struct Stage
{
    Tracks t;
    const double* r;        // input radii [C + T]
    const double* u;        // input conserved [5][C]
    const double* gin;      // ghost primitives inside / outside [T][5]
    const double* gout;
    double dt;
    int use_plm;
    // RK combination: out = base * b + (in + du) * (1 - b); base null: out = in + du
    const double* r_base;
    const double* u_base;
    double b, b1;
    double* r_out;
    double* u_out;
    // workspace
    double* P;              // [5][C] primitives
    double* G;              // [5][C] radial slopes
    double* rf;             // [6][F] radial flux and contact speed
    double* pf;             // [6][NPmax] polar flux and area
    double* fa;             // [F] radial face areas (radial_kernel), shared by the two cells of each face
    int32_t* pil;           // [NPmax] merge counters
    int32_t* pir;
    int64_t np_max;
    const double* tg;       // [T][TG_N] track geometry (trig_kernel)
    int* failures;
};

__device__ inline int64_t track_of(const int64_t* off, int T, int64_t x)
{
    // largest j with off[j] <= x
    int lo = 0, hi = T - 1;
    while (lo < hi)
    {
        const int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= x) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ inline int64_t face_offset(const Tracks& t, int j) { return t.co[j] + j; }
__device__ inline int64_t polar_offset(const Tracks& t, int j) { return t.co[j] + t.co[j + 1] - t.co[1] + j; }

// sedov::cell_volume / face_area (scheme_sedov2d.cpp:40-62)
__device__ inline double cell_volume_cos(double r0, double r1, double c0, double c1)
{
    const double dcost = -(c1 - c0);
    return 2.0 * M_PI * (r1 * r1 * r1 - r0 * r0 * r0) / 3.0 * dcost;
}

// face_area (scheme_sedov2d.cpp) from the sines and cosines of the two polar
// angles; the reference's pow(x, 0.5) is the correctly rounded square root.
__device__ inline double face_area(double r0, double r1, double s0, double c0, double s1, double c1)
{
    const double R0 = r0 * s0, R1 = r1 * s1;
    const double z0 = r0 * c0, z1 = r1 * c1;
    const double dR = R1 - R0, dz = z1 - z0;
    return M_PI * (R0 + R1) * sqrt(dR * dR + dz * dz);
}

// Track geometry, the same for every cell of a track and every stage,
// [T][TG_N]: sin and cos of both polar bounds, the cotangent of the track
// centre q_j = (t0 + t1)/2, q_j itself, and the reciprocal centre spacings
// 1/(q_j - q_{j-1}) and 1/(q_{j+1} - q_{j-1}) of the theta PLM (zero where a
// neighbour is missing).
enum { TG_S0 = 0, TG_C0 = 1, TG_S1 = 2, TG_C1 = 3, TG_COT = 4, TG_QC = 5, TG_IPREV = 6, TG_ISPAN = 7, TG_N = 8 };

__global__ void trig_kernel(const int T, const double* theta, double* tg)
{
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < T; j += gridDim.x * blockDim.x)
    {
        const double t0 = theta[2 * j], t1 = theta[2 * j + 1];
        double* g = tg + TG_N * j;
        g[TG_S0] = sin(t0);
        g[TG_C0] = cos(t0);
        g[TG_S1] = sin(t1);
        g[TG_C1] = cos(t1);
        g[TG_COT] = tan(M_PI_2 - 0.5 * (t0 + t1));
        auto qc = [&](int k) { return 0.5 * (theta[2 * k] + theta[2 * k + 1]); };
        const double q = qc(j);
        g[TG_QC] = q;
        g[TG_IPREV] = j >= 1 ? 1.0 / (q - qc(j - 1)) : 0.0;
        g[TG_ISPAN] = j >= 1 && j + 1 < T ? 1.0 / (qc(j + 1) - qc(j - 1)) : 0.0;
    }
}

// plm_gradient_scalar_t on coordinates (scheme_plm_gradient.hpp:44-67), with
// the reciprocal coordinate spacings il = 1/(x0 - xl), ib = 1/(xr - xl),
// ir = 1/(xr - x0) taken once for all five components (FP64 division is the
// slowest FP64 operation here; the products differ from the quotients by an
// ulp).
// The limiter itself runs on the integer pipes: the magnitudes of doubles
// order as their bit patterns, and the result is the smallest magnitude with
// the common sign, or zero where the signs differ (the reference's
// 0.25 |sa + sb| (sa + sc) min(...) form, without six FP64 operations).
__device__ inline double plm_r(double il, double ib, double ir, double yl, double y0, double yr, double theta)
{
    const double a = (y0 - yl) * il * theta;
    const double b = (yr - yl) * ib;
    const double c = (yr - y0) * ir * theta;
    const long long ba = __double_as_longlong(a), bb = __double_as_longlong(b), bc = __double_as_longlong(c);
    const long long mask = 0x7FFFFFFFFFFFFFFFLL;
    const long long m = min(min(ba & mask, bb & mask), bc & mask);
    return ((ba ^ bb) | (ba ^ bc)) < 0 ? 0.0 : __longlong_as_double(m | (ba & ~mask));
}

__device__ inline double comp(const SPrim<double>& p, int k) { return k == 0 ? p.rho : (k == 4 ? p.p : p.u[k - 1]); }
__device__ inline void set_comp(SPrim<double>& p, int k, double v)
{
    if (k == 0) p.rho = v; else if (k == 4) p.p = v; else p.u[k - 1] = v;
}

__device__ inline SPrim<double> load_prim(const double* P, int64_t C, int64_t c)
{
    SPrim<double> p;
    for (int k = 0; k < 5; ++k) set_comp(p, k, P[k * C + c]);
    return p;
}

__device__ inline SPrim<double> load_ghost(const double* g, int j)
{
    SPrim<double> p;
    for (int k = 0; k < 5; ++k) set_comp(p, k, g[5 * j + k]);
    return p;
}

// the radial slope of cell i (local) of track j: zero at both ends
__device__ inline void load_slope(const Stage& S, int64_t c, double g[5])
{
    for (int k = 0; k < 5; ++k) g[k] = S.G[k * S.t.C + c];
}

__device__ inline void radial_slope(const Stage& S, int j, int64_t i, int64_t n, double g[5])
{
    for (int k = 0; k < 5; ++k) g[k] = 0.0;
    if (i <= 0 || i + 1 >= n) return;
    const int64_t c = S.t.co[j] + i, f = face_offset(S.t, j) + i;
    const double* r = S.r + f;
    const double xl = 0.5 * (r[-1] + r[0]), x0 = 0.5 * (r[0] + r[1]), xr = 0.5 * (r[1] + r[2]);
    const double il = 1.0 / (x0 - xl), ib = 1.0 / (xr - xl), ir = 1.0 / (xr - x0);
    const double th = S.use_plm ? 1.0 : 0.0;
    const int64_t C = S.t.C;
    for (int k = 0; k < 5; ++k)
        g[k] = plm_r(il, ib, ir, S.P[k * C + c - 1], S.P[k * C + c], S.P[k * C + c + 1], th);
}

// One side of a face: conserved state, flux and outer wavespeeds along axis
// (conserved_density, flux, outer_wavespeeds: physics_srhd.hpp:182-195,
// 291-324) from one reciprocal square root for the Lorentz factor and its
// inverse, one reciprocal for the specific enthalpy and the sound speed, and
// one of the wavespeed denominator: two FP64 divisions and two square roots
// where the term-by-term form takes nine and four.
struct Side
{
    double u[5], f[5];
    double vn, am, ap;
};

__device__ inline void side_of(const SPrim<double>& p, int axis, Side& s)
{
    const double gm = kGamma;
    const double ch = 1.0 + 1.0 / (gm - 1.0);            // enthalpy_density's 1 + 1/(gamma - 1)
    const double uu = p.u[0] * p.u[0] + p.u[1] * p.u[1] + p.u[2] * p.u[2];
    const double iW = rsqrt(1.0 + uu);                  // 1/W, and W = (1 + uu)/W
    const double W = (1.0 + uu) * iW;
    const double vn = p.u[axis] * iW;
    const double e = p.rho + p.p * ch;                   // rho c^2 + p gamma / (gamma - 1)
    const double ire = 1.0 / (p.rho * e);                // h = e / rho and a2 = gamma p / e from one reciprocal
    const double h = e * e * ire;
    const double D = p.rho * W;
    s.u[0] = D;
    for (int k = 0; k < 3; ++k) s.u[1 + k] = D * h * p.u[k];
    s.u[4] = D * (h * W - 1.0) - p.p;
    for (int k = 0; k < 5; ++k) s.f[k] = vn * s.u[k];
    s.f[1 + axis] += p.p;
    s.f[4] += p.p * vn;
    const double a2 = gm * p.p * p.rho * ire;
    const double bb = uu * iW * iW;                      // uu / (1 + uu)
    const double disc = a2 * (1.0 - bb) * (1.0 - bb * a2 - vn * vn * (1.0 - a2));
    const double k0 = sqrt(disc);
    const double iden = 1.0 / (1.0 - bb * a2);
    const double vna = vn * (1.0 - a2);
    s.vn = vn;
    s.am = (vna - k0) * iden;
    s.ap = (vna + k0) * iden;
}

// The HLLC modes of riemann_solver (physics_srhd.hpp:351-487) along axis:
// FIXED (face speed 0), MOVING (face speed w), ACROSS (the left star flux
// with the contact speed, which is returned in *contact). Returns 1 where the
// reference throws (NaN contact speed or beyond 1e3). Divisions by the same
// denominator (the HLL fan width, each star state's s - s*) are one
// reciprocal and products.
enum { FIXED = 0, MOVING = 1, ACROSS = 2 };

__device__ inline int hllc_mode(const SPrim<double>& pl, const SPrim<double>& pr, int axis, int mode, double w,
                                double F[5], double* contact)
{
    Side L, R;
    side_of(pl, axis, L);
    side_of(pr, axis, R);
    const double ar = fmax(L.ap, R.ap);
    const double al = fmin(L.am, R.am);
    const double ifan = 1.0 / (ar - al);
    double u_hll[5], f_hll[5];
    for (int k = 0; k < 5; ++k)
    {
        u_hll[k] = (ar * R.u[k] - al * L.u[k] + (L.f[k] - R.f[k])) * ifan;
        f_hll[k] = (ar * L.f[k] - al * R.f[k] - (L.u[k] - R.u[k]) * ar * al) * ifan;
    }
    const double ue_hll = u_hll[4] + u_hll[0];
    const double fe_hll = f_hll[4] + f_hll[0];
    const double um_hll = u_hll[1 + axis];
    const double fm_hll = f_hll[1 + axis];
    const double a = fe_hll;
    const double b = -fm_hll - ue_hll;
    const double c = um_hll;
    const double d = b * b - 4.0 * a * c;
    const double as = d < 0.0 ? 0.0 : (fabs(a) > 1e-8 ? (-b - sqrt(d)) / (2.0 * a) : -c / b);
    if (isnan(as) || as < -1e3 || as > 1e3)
    {
        for (int k = 0; k < 5; ++k) F[k] = 0.0;
        if (contact) *contact = 0.0;
        return 1;
    }
    const double ps = -fe_hll * as + fm_hll;
    auto star = [&](const Side& q, const SPrim<double>& p, double s, double face) {
        const double v = q.vn;
        const double e = q.u[4] + q.u[0];
        const double m = q.u[1 + axis];
        const double sv = s - v;
        const double isa = 1.0 / (s - as);
        const double es = (e * sv + ps * as - p.p * v) * isa;
        const double ms = (m * sv + ps - p.p) * isa;
        const double Ds = q.u[0] * sv * isa;
        double us[5];
        us[0] = Ds;
        for (int k = 0; k < 3; ++k) us[1 + k] = k == axis ? ms : q.u[1 + k] * sv * isa;
        us[4] = es - Ds;
        for (int k = 0; k < 5; ++k) F[k] = q.f[k] + s * (us[k] - q.u[k]) - face * us[k];
    };
    if (mode == ACROSS)
    {
        star(L, pl, al, as);
        if (contact) *contact = as;
        return 0;
    }
    if (mode == MOVING)
    {
        if (w <= al) { for (int k = 0; k < 5; ++k) F[k] = L.f[k] - w * L.u[k]; return 0; }
        if (w >= ar) { for (int k = 0; k < 5; ++k) F[k] = R.f[k] - w * R.u[k]; return 0; }
        if (w <= as) star(L, pl, al, w);
        else star(R, pr, ar, w);
        return 0;
    }
    if (0.0 <= al) { for (int k = 0; k < 5; ++k) F[k] = L.f[k]; return 0; }
    if (0.0 >= ar) { for (int k = 0; k < 5; ++k) F[k] = R.f[k]; return 0; }
    if (0.0 <= as) star(L, pl, al, 0.0);
    else star(R, pr, ar, 0.0);
    return 0;
}

__device__ inline void count_failure(const Stage& S, int bad)
{
    if (bad && S.failures) atomicAdd(S.failures, bad);
}

// ---------------------------------------------------------------- kernels
__global__ void __launch_bounds__(256) prim_kernel(const Stage S)
{
    const int64_t C = S.t.C;
    for (int64_t c = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; c < C; c += int64_t(gridDim.x) * blockDim.x)
    {
        const int j = int(track_of(S.t.co, S.t.T, c));
        const int64_t i = c - S.t.co[j];
        const double* r = S.r + face_offset(S.t, j) + i;
        const double dv = cell_volume_cos(r[0], r[1], S.tg[TG_N * j + TG_C0], S.tg[TG_N * j + TG_C1]);
        const double idv = 1.0 / dv;
        srhd::Zone z{S.u[c] * idv, S.u[C + c] * idv, S.u[2 * C + c] * idv, S.u[3 * C + c] * idv,
                     S.u[4 * C + c] * idv};
        double prim[5] = {0, 0, 0, 0, 0};
        int it = 0;
        // the reference's iteration from p = 0 with its stopping rule, its
        // update as three reciprocals and an inverse square root; a zone it
        // does not bring home takes the term-by-term iteration
        int st = srhd::newton_fast(z, kGamma, kFloor, 0.0, 50, prim, it);
        if (st != 0) st = srhd::newton(z, kGamma, kFloor, 0.0, 50, prim, it);
        if (st != 0)
            for (int k = 0; k < 5; ++k) prim[k] = 0.0;
        count_failure(S, st != 0);
        for (int k = 0; k < 5; ++k) S.P[k * C + c] = prim[k];
    }
}

// radial_gradient (scheme_sedov2d.cpp:188-203)
__global__ void __launch_bounds__(256) grad_kernel(const Stage S)
{
    const int64_t C = S.t.C;
    for (int64_t c = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; c < C; c += int64_t(gridDim.x) * blockDim.x)
    {
        const int j = int(track_of(S.t.co, S.t.T, c));
        double g[5];
        radial_slope(S, j, c - S.t.co[j], S.t.co[j + 1] - S.t.co[j], g);
        for (int k = 0; k < 5; ++k) S.G[k * C + c] = g[k];
    }
}

__global__ void __launch_bounds__(256) radial_kernel(const Stage S)
{
    const int64_t C = S.t.C, F = C + S.t.T;
    for (int64_t f = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; f < F; f += int64_t(gridDim.x) * blockDim.x)
    {
        // faces of track j: [co[j] + j, co[j+1] + j], i.e. face offsets co[j] + j
        int lo = 0, hi = S.t.T - 1;
        while (lo < hi)
        {
            const int mid = (lo + hi + 1) >> 1;
            if (S.t.co[mid] + mid <= f) lo = mid; else hi = mid - 1;
        }
        const int j = lo;
        const int64_t n = S.t.co[j + 1] - S.t.co[j];
        const int64_t i = f - face_offset(S.t, j);
        const int64_t c0 = S.t.co[j];
        double flux[5], speed = 0.0;
        int bad = 0;
        if (i == 0)
        {
            // inner_bc (problems/sedov2d.cpp:563-574)
            const SPrim<double> front = load_prim(S.P, C, c0);
            speed = fmin(1.0 * front.u[0] / srhd::lorentz_factor(front), 0.0);
            bad = hllc_mode(load_ghost(S.gin, j), front, 0, MOVING, speed, flux, nullptr);
        }
        else if (i == n)
        {
            // outer_bc (problems/sedov2d.cpp:576-587)
            const SPrim<double> ghost = load_ghost(S.gout, j);
            speed = 1.0 * ghost.u[0] / srhd::lorentz_factor(ghost);
            bad = hllc_mode(load_prim(S.P, C, c0 + n - 1), ghost, 0, MOVING, speed, flux, nullptr);
        }
        else
        {
            // radial_godunov_data (scheme_sedov2d.cpp:208-230)
            double gl[5], gr[5];
            load_slope(S, c0 + i - 1, gl);
            load_slope(S, c0 + i, gr);
            const double drl = S.r[f] - S.r[f - 1], drr = S.r[f + 1] - S.r[f];
            SPrim<double> pl = load_prim(S.P, C, c0 + i - 1), pr = load_prim(S.P, C, c0 + i);
            for (int k = 0; k < 5; ++k)
            {
                set_comp(pl, k, comp(pl, k) + 0.5 * gl[k] * drl);
                set_comp(pr, k, comp(pr, k) - 0.5 * gr[k] * drr);
            }
            bad = hllc_mode(pl, pr, 0, ACROSS, 0.0, flux, &speed);
        }
        count_failure(S, bad);
        for (int k = 0; k < 5; ++k) S.rf[k * F + f] = flux[k];
        S.rf[5 * F + f] = speed;
        {
            const double* g = S.tg + TG_N * j;
            S.fa[f] = face_area(S.r[f], S.r[f], g[TG_S0], g[TG_C0], g[TG_S1], g[TG_C1]);
        }
        // delta_face_positions + the RK combination
        const double moved = S.r[f] + speed * S.dt;
        S.r_out[f] = S.r_base ? S.r_base[f] * S.b + moved * S.b1 : moved;
    }
}

// Face radii are positive, so they order as their bit patterns: the merge
// path and the samples compare them on the integer pipes, which leaves the
// FP64 pipe (the bound of these kernels) to the arithmetic.
__device__ inline long long rbits(double r) { return __double_as_longlong(r); }

// sedov::sample (scheme_sedov2d.cpp:235-253) on track j (or the fallback)
__device__ inline SPrim<double> sample(const Stage& S, int j, double r, int64_t index, const SPrim<double>& fallback)
{
    const int64_t n = S.t.co[j + 1] - S.t.co[j];
    const double* rf = S.r + face_offset(S.t, j);
    const long long rb = rbits(r);
    if (rb <= rbits(rf[0]) || rb >= rbits(rf[n])) return fallback;
    index = min(index, n);
    // the walk of the reference from the hint; r lies strictly inside the
    // track, so it ends within [0, n - 1]; the bound only guards bad input
    for (int64_t guard = 0; guard <= n && rb < rbits(rf[index]); ++guard) --index;
    for (int64_t guard = 0; guard <= n && rb > rbits(rf[index + 1]); ++guard) ++index;
    index = max(int64_t(0), min(index, n - 1));
    const double rc = 0.5 * (rf[index] + rf[index + 1]);
    const int64_t c = S.t.co[j] + index;
    double g[5];
    load_slope(S, c, g);
    SPrim<double> out;
    for (int k = 0; k < 5; ++k) set_comp(out, k, S.P[k * S.t.C + c] + g[k] * (r - rc));
    return out;
}

__global__ void __launch_bounds__(256) polar_kernel(const Stage S)
{
    const int T = S.t.T;
    if (T < 2) return;
    const int64_t NP = polar_offset(S.t, T - 1);
    for (int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; p < NP; p += int64_t(gridDim.x) * blockDim.x)
    {
        int lo = 0, hi = T - 2;
        while (lo < hi)
        {
            const int mid = (lo + hi + 1) >> 1;
            if (polar_offset(S.t, mid) <= p) lo = mid; else hi = mid - 1;
        }
        const int j = lo;
        const int64_t m = p - polar_offset(S.t, j);           // face m of interface j | j + 1
        const double* L = S.r + face_offset(S.t, j);
        const double* R = S.r + face_offset(S.t, j + 1);
        const int64_t nl = S.t.co[j + 1] - S.t.co[j] + 1, nr = S.t.co[j + 2] - S.t.co[j + 1] + 1;
        // merge path: a = how many of L are among the first m + 1 merged radii (L first on ties)
        const int64_t d = m + 1;
        int64_t a = max(int64_t(0), d - nr), b = min(d, nl);
        while (a < b)
        {
            const int64_t mid = (a + b) >> 1;
            if (rbits(L[mid]) <= rbits(R[d - mid - 1])) a = mid + 1; else b = mid;
        }
        const int64_t il = a - 1, ir = m - a;
        // the larger radius of the two trailing faces and the smaller of the
        // two leading ones (a missing face is -inf / +inf), compared as bits
        const double tl = il >= 0 ? L[il] : -INFINITY, tr = ir >= 0 ? R[ir] : -INFINITY;
        const double ll = a < nl ? L[a] : INFINITY, lr = m + 1 - a < nr ? R[m + 1 - a] : INFINITY;
        const double trailing = rbits(tl) >= rbits(tr) ? tl : tr;
        const double leading = rbits(ll) <= rbits(lr) ? ll : lr;
        S.pil[p] = int32_t(il);
        S.pir[p] = int32_t(ir);
        const bool valid = il >= 0 && il + 1 < nl && ir >= 0 && ir + 1 < nr;
        double flux[5] = {0, 0, 0, 0, 0}, da = 0.0;
        if (valid)
        {
            const double ql = S.t.theta[2 * j + 1], qr = S.t.theta[2 * (j + 1)];
            const double rf = 0.5 * (trailing + leading);
            const SPrim<double> none{0.0, {0.0, 0.0, 0.0}, 0.0};
            SPrim<double> pl, pr;
            if (!S.use_plm || j == 0 || j + 2 >= T)
            {
                pl = sample(S, j, rf, il, none);
                pr = sample(S, j + 1, rf, ir, none);
            }
            else
            {
                // track centres and reciprocal spacings from the geometry table
                const double* g1 = S.tg + TG_N * j;
                const double* g2 = g1 + TG_N;
                const double q1 = g1[TG_QC], q2 = g2[TG_QC];
                const SPrim<double> p1 = sample(S, j, rf, il, none);
                const SPrim<double> p2 = sample(S, j + 1, rf, ir, none);
                const SPrim<double> p0 = sample(S, j - 1, rf, il, p1);
                const SPrim<double> p3 = sample(S, j + 2, rf, ir, p2);
                const double i10 = g1[TG_IPREV], i20 = g1[TG_ISPAN], i21 = g2[TG_IPREV];
                const double i31 = g2[TG_ISPAN], i32 = g2[TG_N + TG_IPREV];
                for (int k = 0; k < 5; ++k)
                {
                    const double cl = plm_r(i10, i20, i21, comp(p0, k), comp(p1, k), comp(p2, k), 1.0);
                    const double cr = plm_r(i21, i31, i32, comp(p1, k), comp(p2, k), comp(p3, k), 1.0);
                    set_comp(pl, k, comp(p1, k) + (ql - q1) * cl);
                    set_comp(pr, k, comp(p2, k) + (qr - q2) * cr);
                }
            }
            count_failure(S, hllc_mode(pl, pr, 1, FIXED, 0.0, flux, nullptr));
            da = face_area(trailing, leading, S.tg[TG_N * j + TG_S1], S.tg[TG_N * j + TG_C1],
                           S.tg[TG_N * (j + 1) + TG_S0], S.tg[TG_N * (j + 1) + TG_C0]);
        }
        for (int k = 0; k < 5; ++k) S.pf[k * S.np_max + p] = flux[k];
        S.pf[5 * S.np_max + p] = da;
    }
}

// first index in [lo, hi) whose counter is >= v (counters are nondecreasing)
__device__ inline int64_t lower_bound(const int32_t* a, int64_t lo, int64_t hi, int64_t v)
{
    while (lo < hi)
    {
        const int64_t mid = (lo + hi) >> 1;
        if (a[mid] < v) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__global__ void __launch_bounds__(256) update_kernel(const Stage S)
{
    const int64_t C = S.t.C, F = C + S.t.T;
    const int T = S.t.T;
    for (int64_t c = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; c < C; c += int64_t(gridDim.x) * blockDim.x)
    {
        const int j = int(track_of(S.t.co, T, c));
        const int64_t n = S.t.co[j + 1] - S.t.co[j];
        const int64_t i = c - S.t.co[j];
        const int64_t f = face_offset(S.t, j) + i;
        const double* g = S.tg + TG_N * j;
        const double r0 = S.r[f], r1 = S.r[f + 1];
        const double da0 = S.fa[f], da1 = S.fa[f + 1];    // face_area of both radial faces (radial_kernel)
        const double dv = cell_volume_cos(r0, r1, g[TG_C0], g[TG_C1]);
        // polar fluxes binned on this cell, in face order (mesh::bin_values)
        double gl[5] = {0, 0, 0, 0, 0}, gr[5] = {0, 0, 0, 0, 0};
        if (j > 0)
        {
            // interface j-1 | j: this track is the right side, binned by ir
            const int64_t p0 = polar_offset(S.t, j - 1), p1 = polar_offset(S.t, j);
            const int64_t nl = S.t.co[j] - S.t.co[j - 1] + 1;
            for (int64_t p = lower_bound(S.pir, p0, p1, i); p < p1 && S.pir[p] == i; ++p)
            {
                const int64_t il = S.pil[p];
                if (il < 0 || il + 1 >= nl) continue;
                const double da = S.pf[5 * S.np_max + p];
                for (int k = 0; k < 5; ++k) gl[k] = gl[k] + S.pf[k * S.np_max + p] * da;
            }
        }
        if (j + 1 < T)
        {
            // interface j | j+1: this track is the left side, binned by il
            const int64_t p0 = polar_offset(S.t, j), p1 = polar_offset(S.t, j + 1);
            const int64_t nr = S.t.co[j + 2] - S.t.co[j + 1] + 1;
            for (int64_t p = lower_bound(S.pil, p0, p1, i); p < p1 && S.pil[p] == i; ++p)
            {
                const int64_t ir = S.pir[p];
                if (ir < 0 || ir + 1 >= nr) continue;
                const double da = S.pf[5 * S.np_max + p];
                for (int k = 0; k < 5; ++k) gr[k] = gr[k] + S.pf[k * S.np_max + p] * da;
            }
        }
        // spherical_geometry_source_terms (physics_srhd.hpp:330-345)
        const SPrim<double> p = load_prim(S.P, C, c);
        const double rc = 0.5 * (r0 + r1);
        const double cotq = g[TG_COT];
        const double ur = p.u[0], uq = p.u[1], up = p.u[2], pg = p.p;
        const double H0 = srhd::enthalpy_density(p, kGamma);
        const double irc = 1.0 / rc;
        const double src[5] = {0.0, (2.0 * pg + H0 * (uq * uq + up * up)) * irc,
                               (cotq * pg + H0 * (up * up * cotq - ur * uq)) * irc, -up * H0 * (ur + uq * cotq) * irc,
                               0.0};
        for (int k = 0; k < 5; ++k)
        {
            const double df = S.rf[k * F + f + 1] * da1 - S.rf[k * F + f] * da0;
            const double dg = gr[k] - gl[k];
            const double sc = src[k] * dv;
            const double out = S.u[k * C + c] + (-(df + dg) + sc) * S.dt;
            S.u_out[k * C + c] = S.u_base ? S.u_base[k * C + c] * S.b + out * S.b1 : out;
        }
        (void)n;
    }
}

__global__ void min_spacing_kernel(Tracks t, const double* r, unsigned long long* out)
{
    double m = INFINITY;
    const int64_t C = t.C;
    for (int64_t c = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; c < C; c += int64_t(gridDim.x) * blockDim.x)
    {
        const int j = int(track_of(t.co, t.T, c));
        const int64_t f = c + j;
        m = fmin(m, r[f + 1] - r[f]);
    }
    for (int o = 16; o > 0; o >>= 1) m = fmin(m, __shfl_xor_sync(0xffffffffu, m, o));
    // positive doubles order as their bit patterns
    if ((threadIdx.x & 31) == 0 && m > 0.0) atomicMin(out, (unsigned long long)__double_as_longlong(m));
}

// ---------------------------------------------------------------- remesh
// sedov::remesh (scheme_sedov2d.cpp:362-412) of every track: one warp per
// track edits a scratch copy (drop the first cell, merge two cells, split a
// cell) with warp-wide shifts, then the new tracks are packed by an offset
// scan. The reference recurses after a drop or a merge with the two aspect
// bounds passed in exchanged order, so each further level runs with them
// exchanged; that is kept.
struct Remesh
{
    int T;
    int64_t C;
    const int64_t* co;
    const double* theta;
    const double* r;
    const double* u;
    double* rs;            // scratch radii: track j at co[j] + 2j, capacity n + 2
    double* us;            // scratch cells: [5][C + T], track j at co[j] + j, capacity n + 1
    int64_t* counts;       // [T] new cell counts
    int64_t* co_out;       // [T + 1]
    double* r_out;
    double* u_out;
    double max_aspect, min_aspect, inner;
    int* failures;
};

// a[k - 1] = a[k] for k in [from, end), ascending chunks of one warp
__device__ inline void warp_shift_left(double* a, int64_t from, int64_t end, int lane)
{
    for (int64_t base = from; base < end; base += 32)
    {
        const int64_t k = base + lane;
        const double v = k < end ? a[k] : 0.0;
        __syncwarp();
        if (k < end) a[k - 1] = v;
        __syncwarp();
    }
}

// a[k + 1] = a[k] for k in [from, end), descending chunks of one warp
__device__ inline void warp_shift_right(double* a, int64_t from, int64_t end, int lane)
{
    for (int64_t top = end; top > from; top -= 32)
    {
        const int64_t k = top - 1 - lane;
        const double v = k >= from ? a[k] : 0.0;
        __syncwarp();
        if (k >= from) a[k + 1] = v;
        __syncwarp();
    }
}

__global__ void remesh_track_kernel(const Remesh M)
{
    const int lane = threadIdx.x & 31;
    const int64_t j = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    if (j >= M.T) return;                                     // uniform per warp
    const int64_t S5 = M.C + M.T;
    int64_t n = M.co[j + 1] - M.co[j];
    double* rf = M.rs + M.co[j] + 2 * j;
    double* uc[5];
    for (int q = 0; q < 5; ++q) uc[q] = M.us + q * S5 + M.co[j] + j;
    for (int64_t k = lane; k <= n; k += 32) rf[k] = M.r[M.co[j] + j + k];
    for (int64_t k = lane; k < n; k += 32)
        for (int q = 0; q < 5; ++q) uc[q][k] = M.u[q * M.C + M.co[j] + k];
    __syncwarp();
    const double dth = M.theta[2 * j + 1] - M.theta[2 * j];
    double amax_b = M.max_aspect, amin_b = M.min_aspect;
    int bad = 0;
    for (int64_t guard = 0; guard < 2 * n + 4; ++guard)
    {
        // aspect dr / (r_c dtheta); nd::argmin / argmax take the first index
        double mn = INFINITY, mx = -INFINITY;
        int64_t imn = 0, imx = 0;
        for (int64_t k = lane; k < n; k += 32)
        {
            const double a = (rf[k + 1] - rf[k]) / ((0.5 * (rf[k] + rf[k + 1])) * dth);
            if (a < mn) { mn = a; imn = k; }
            if (a > mx) { mx = a; imx = k; }
        }
        for (int o = 16; o > 0; o >>= 1)
        {
            const double omn = __shfl_xor_sync(0xffffffffu, mn, o), omx = __shfl_xor_sync(0xffffffffu, mx, o);
            const int64_t oimn = __shfl_xor_sync(0xffffffffu, imn, o), oimx = __shfl_xor_sync(0xffffffffu, imx, o);
            if (omn < mn || (omn == mn && oimn < imn)) { mn = omn; imn = oimn; }
            if (omx > mx || (omx == mx && oimx < imx)) { mx = omx; imx = oimx; }
        }
        if (rf[0] < M.inner)
        {
            if (n < 2) { bad = 1; break; }
            warp_shift_left(rf, 1, n + 1, lane);
            for (int q = 0; q < 5; ++q) warp_shift_left(uc[q], 1, n, lane);
            n -= 1;
            const double t = amax_b; amax_b = amin_b; amin_b = t;
            continue;
        }
        if (mx > amax_b)
        {
            const double mid = 0.5 * (rf[imx] + rf[imx + 1]);
            double half[5];
            for (int q = 0; q < 5; ++q) half[q] = 0.5 * uc[q][imx];
            __syncwarp();
            warp_shift_right(rf, imx + 1, n + 1, lane);
            for (int q = 0; q < 5; ++q) warp_shift_right(uc[q], imx + 1, n, lane);
            if (lane == 0)
            {
                rf[imx + 1] = mid;
                for (int q = 0; q < 5; ++q) uc[q][imx] = uc[q][imx + 1] = half[q];
            }
            __syncwarp();
            n += 1;
            break;
        }
        if (mn < amin_b)
        {
            int64_t e = -1;
            if (imn == 0) e = 1;
            else if (imn + 1 == n) e = imn;
            else
            {
                const double al = (rf[imn] - rf[imn - 1]) / ((0.5 * (rf[imn - 1] + rf[imn])) * dth);
                const double ar = (rf[imn + 2] - rf[imn + 1]) / ((0.5 * (rf[imn + 1] + rf[imn + 2])) * dth);
                if (al <= ar) e = imn;
                else if (al >= ar) e = imn + 1;
            }
            if (e < 0) break;
            if (e + 1 >= n + 1) { bad = 1; break; }
            double merged[5];
            for (int q = 0; q < 5; ++q) merged[q] = uc[q][e - 1] + uc[q][e];
            __syncwarp();
            if (lane == 0)
                for (int q = 0; q < 5; ++q) uc[q][e - 1] = merged[q];
            __syncwarp();
            for (int q = 0; q < 5; ++q) warp_shift_left(uc[q], e + 1, n, lane);
            warp_shift_left(rf, e + 1, n + 1, lane);
            n -= 1;
            const double t = amax_b; amax_b = amin_b; amin_b = t;
            continue;
        }
        break;
    }
    if (lane == 0)
    {
        M.counts[j] = n;
        if (bad && M.failures) atomicAdd(M.failures, 1);
    }
}

// exclusive scan of the new counts into co_out (one block)
__global__ void remesh_scan_kernel(const Remesh M)
{
    __shared__ int64_t part[1024];
    const int t = threadIdx.x, nt = blockDim.x;
    const int64_t per = (M.T + nt - 1) / nt;
    const int64_t a = t * per, b = min(int64_t(M.T), a + per);
    int64_t sum = 0;
    for (int64_t k = a; k < b; ++k) sum += M.counts[k];
    part[t] = sum;
    __syncthreads();
    if (t == 0)
    {
        int64_t run = 0;
        for (int k = 0; k < nt; ++k) { const int64_t v = part[k]; part[k] = run; run += v; }
        M.co_out[M.T] = run;
    }
    __syncthreads();
    int64_t run = part[t];
    for (int64_t k = a; k < b; ++k) { M.co_out[k] = run; run += M.counts[k]; }
}

__global__ void remesh_pack_kernel(const Remesh M)
{
    const int lane = threadIdx.x & 31;
    const int64_t j = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    if (j >= M.T) return;
    const int64_t S5 = M.C + M.T, Cn = M.co_out[M.T];
    const int64_t n = M.co_out[j + 1] - M.co_out[j];
    const double* rf = M.rs + M.co[j] + 2 * j;
    for (int64_t k = lane; k <= n; k += 32) M.r_out[M.co_out[j] + j + k] = rf[k];
    for (int64_t k = lane; k < n; k += 32)
        for (int q = 0; q < 5; ++q) M.u_out[q * Cn + M.co_out[j] + k] = M.us[q * S5 + M.co[j] + j + k];
}

// ---------------------------------------------------------------- host
struct Workspace
{
    double* P;
    double* G;
    double* rf;
    double* pf;
    int32_t* pil;
    int32_t* pir;
    double* r_stage[2];
    double* u_stage[2];
    double* tg;
    double* fa;
    int* failures;
    int64_t np_max;
};

int64_t np_bound(int T, int64_t C) { return 2 * C + T; }

int64_t workspace_bytes(int T, int64_t C)
{
    const int64_t F = C + T, NP = np_bound(T, C);
    auto al = [](int64_t b) { return (b + 255) / 256 * 256; };
    return 2 * al(5 * C * 8) + al(6 * F * 8) + al(6 * NP * 8) + 2 * al(NP * 4) + 2 * al(F * 8) + 2 * al(5 * C * 8) +
           al(TG_N * int64_t(T) * 8) + al(F * 8) + 256 + 256;
}

Workspace carve(void* base, int T, int64_t C)
{
    const int64_t F = C + T, NP = np_bound(T, C);
    char* p = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(base) + 255) & ~uintptr_t(255));
    auto take = [&](int64_t bytes) { char* q = p; p += (bytes + 255) / 256 * 256; return q; };
    Workspace w;
    w.P = reinterpret_cast<double*>(take(5 * C * 8));
    w.G = reinterpret_cast<double*>(take(5 * C * 8));
    w.rf = reinterpret_cast<double*>(take(6 * F * 8));
    w.pf = reinterpret_cast<double*>(take(6 * NP * 8));
    w.pil = reinterpret_cast<int32_t*>(take(NP * 4));
    w.pir = reinterpret_cast<int32_t*>(take(NP * 4));
    for (int s = 0; s < 2; ++s) w.r_stage[s] = reinterpret_cast<double*>(take(F * 8));
    for (int s = 0; s < 2; ++s) w.u_stage[s] = reinterpret_cast<double*>(take(5 * C * 8));
    w.tg = reinterpret_cast<double*>(take(TG_N * int64_t(T) * 8));
    w.fa = reinterpret_cast<double*>(take(F * 8));
    w.failures = reinterpret_cast<int*>(take(256));
    w.np_max = NP;
    return w;
}

inline int blocks_for(int64_t n) { return int(std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16))); }

int launch_trig(const Tracks& t, double* tg, cudaStream_t s)
{
    trig_kernel<<<blocks_for(t.T), 256, 0, s>>>(t.T, t.theta, tg);
    return launch_status("sedov trig_kernel");
}

int run_stage(Stage S, cudaStream_t s)
{
    const int64_t C = S.t.C, F = C + S.t.T;
    prim_kernel<<<blocks_for(C), 256, 0, s>>>(S);
    if (int r = launch_status("sedov prim_kernel")) return r;
    grad_kernel<<<blocks_for(C), 256, 0, s>>>(S);
    if (int r = launch_status("sedov grad_kernel")) return r;
    radial_kernel<<<blocks_for(F), 256, 0, s>>>(S);
    if (int r = launch_status("sedov radial_kernel")) return r;
    polar_kernel<<<blocks_for(S.np_max), 256, 0, s>>>(S);
    if (int r = launch_status("sedov polar_kernel")) return r;
    update_kernel<<<blocks_for(C), 256, 0, s>>>(S);
    return launch_status("sedov update_kernel");
}

int check_tracks(int T, int64_t C, const int64_t* co, const double* theta)
{
    MARA_REQUIRE(T >= 1 && T <= (1 << 24), "sedov: track_count must be in [1, 2^24]");
    MARA_REQUIRE(C >= 2 * int64_t(T) && C + T < (int64_t(1) << 31) / 3,
                 "sedov: cells must be at least 2 per track and fewer than 2^31/3 - track_count");
    MARA_REQUIRE(co && theta, "sedov: null track buffer");
    return MARA_OK;
}

} // namespace sedov
} // namespace mara

using namespace mara;
using namespace mara::sedov;

extern "C" {

int64_t mara_sedov_workspace_bytes(int32_t track_count, int64_t cells)
{
    if (track_count < 1 || cells < 2 * int64_t(track_count)) return -1;
    return workspace_bytes(track_count, cells);
}

int mara_sedov_stage(int32_t track_count, int64_t cells, const int64_t* cell_offset, const double* theta,
                     const double* radii, const double* u, const double* ghost_in, const double* ghost_out, double dt,
                     int32_t use_plm, double* radii_out, double* u_out, double* prim, double* grad, double* radial,
                     double* polar, int32_t* polar_index, void* workspace, int32_t* failures, void* stream)
{
    if (int r = check_tracks(track_count, cells, cell_offset, theta)) return r;
    MARA_REQUIRE(radii && u && ghost_in && ghost_out && radii_out && u_out && workspace, "mara_sedov_stage: null buffer");
    MARA_REQUIRE(radii_out != radii && u_out != u, "mara_sedov_stage: outputs must not alias inputs");
    cudaStream_t s = as_stream(stream);
    Workspace w = carve(workspace, track_count, cells);
    Stage S{};
    S.t = Tracks{track_count, cells, cell_offset, theta};
    S.r = radii;
    S.u = u;
    S.gin = ghost_in;
    S.gout = ghost_out;
    S.dt = dt;
    S.use_plm = use_plm != 0;
    S.r_out = radii_out;
    S.u_out = u_out;
    S.P = prim ? prim : w.P;
    S.G = grad ? grad : w.G;
    S.rf = radial ? radial : w.rf;
    S.pf = polar ? polar : w.pf;
    S.pil = polar_index ? polar_index : w.pil;
    S.pir = polar_index ? polar_index + w.np_max : w.pir;
    S.np_max = w.np_max;
    S.tg = w.tg;
    S.fa = w.fa;
    S.failures = failures;
    if (int r = launch_trig(S.t, w.tg, s)) return r;
    return run_stage(S, s);
}

int mara_sedov_advance(int32_t track_count, int64_t cells, const int64_t* cell_offset, const double* theta,
                       double* radii, double* u, const double* ghost_in, const double* ghost_out, double dt,
                       int32_t rk_order, int32_t use_plm, void* workspace, int32_t* failures, void* stream)
{
    if (int r = check_tracks(track_count, cells, cell_offset, theta)) return r;
    MARA_REQUIRE(radii && u && ghost_in && ghost_out && workspace, "mara_sedov_advance: null buffer");
    MARA_REQUIRE(rk_order >= 1 && rk_order <= 3, "mara_sedov_advance: rk_order must be 1, 2 or 3");
    cudaStream_t s = as_stream(stream);
    const int T = track_count;
    Workspace w = carve(workspace, T, cells);
    Stage base{};
    base.t = Tracks{T, cells, cell_offset, theta};
    base.dt = dt;
    base.use_plm = use_plm != 0;
    base.P = w.P;
    base.G = w.G;
    base.rf = w.rf;
    base.pf = w.pf;
    base.pil = w.pil;
    base.pir = w.pir;
    base.np_max = w.np_max;
    base.tg = w.tg;
    base.fa = w.fa;
    base.failures = failures;
    if (int r = launch_trig(base.t, w.tg, s)) return r;
    auto stage = [&](int k, const double* rin, const double* uin, double* rout, double* uout, const double* rb,
                     const double* ub, double b, double b1) {
        Stage S = base;
        S.r = rin;
        S.u = uin;
        S.gin = ghost_in + 5 * int64_t(T) * k;
        S.gout = ghost_out + 5 * int64_t(T) * k;
        S.r_out = rout;
        S.u_out = uout;
        S.r_base = rb;
        S.u_base = ub;
        S.b = b;
        S.b1 = b1;
        return run_stage(S, s);
    };
    double* ra = w.r_stage[0];
    double* ua = w.u_stage[0];
    double* rb = w.r_stage[1];
    double* ub = w.u_stage[1];
    const int64_t F = cells + T;
    if (rk_order == 1)
    {
        if (int r = stage(0, radii, u, ra, ua, nullptr, nullptr, 0, 0)) return r;
    }
    else if (rk_order == 2)
    {
        // u1 = L(u0); u = u0 / 2 + L(u1) / 2 (app_control.hpp:178-183)
        if (int r = stage(0, radii, u, ra, ua, nullptr, nullptr, 0, 0)) return r;
        if (int r = stage(1, ra, ua, rb, ub, radii, u, 1.0 / 2, 1.0 / 2)) return r;
        ra = rb;
        ua = ub;
    }
    else
    {
        // u1 = L(u0); u2 = 3/4 u0 + 1/4 L(u1); u = 1/3 u0 + 2/3 L(u2) (app_control.hpp:184-190)
        if (int r = stage(0, radii, u, ra, ua, nullptr, nullptr, 0, 0)) return r;
        if (int r = stage(1, ra, ua, rb, ub, radii, u, 3.0 / 4, 1.0 / 4)) return r;
        if (int r = stage(2, rb, ub, ra, ua, radii, u, 1.0 / 3, 2.0 / 3)) return r;
    }
    MARA_CUDA(cudaMemcpyAsync(radii, ra, F * sizeof(double), cudaMemcpyDeviceToDevice, s));
    MARA_CUDA(cudaMemcpyAsync(u, ua, 5 * cells * sizeof(double), cudaMemcpyDeviceToDevice, s));
    return MARA_OK;
}

int64_t mara_sedov_remesh_workspace_bytes(int32_t track_count, int64_t cells)
{
    if (track_count < 1 || cells < 2 * int64_t(track_count)) return -1;
    const int64_t T = track_count;
    return (cells + 2 * T) * 8 + 5 * (cells + T) * 8 + T * 8 + 3 * 256;
}

int mara_sedov_remesh(int32_t track_count, int64_t cells, const int64_t* cell_offset, const double* theta,
                      const double* radii, const double* u, double max_aspect, double min_aspect, double inner_radius,
                      int64_t* cell_offset_out, double* radii_out, double* u_out, int64_t* cells_out, void* workspace,
                      int32_t* failures, void* stream)
{
    if (int r = check_tracks(track_count, cells, cell_offset, theta)) return r;
    MARA_REQUIRE(radii && u && cell_offset_out && radii_out && u_out && cells_out && workspace,
                 "mara_sedov_remesh: null buffer");
    MARA_REQUIRE(radii_out != radii && u_out != u && cell_offset_out != cell_offset,
                 "mara_sedov_remesh: outputs must not alias inputs");
    cudaStream_t s = as_stream(stream);
    const int64_t T = track_count;
    char* p = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
    Remesh M{};
    M.T = track_count;
    M.C = cells;
    M.co = cell_offset;
    M.theta = theta;
    M.r = radii;
    M.u = u;
    M.rs = reinterpret_cast<double*>(p);
    p += ((cells + 2 * T) * 8 + 255) / 256 * 256;
    M.us = reinterpret_cast<double*>(p);
    p += (5 * (cells + T) * 8 + 255) / 256 * 256;
    M.counts = reinterpret_cast<int64_t*>(p);
    M.co_out = cell_offset_out;
    M.r_out = radii_out;
    M.u_out = u_out;
    M.max_aspect = max_aspect;
    M.min_aspect = min_aspect;
    M.inner = inner_radius;
    M.failures = failures;
    const int warps_per_block = 8;
    const int blocks = int((T + warps_per_block - 1) / warps_per_block);
    remesh_track_kernel<<<blocks, warps_per_block * 32, 0, s>>>(M);
    if (int r = launch_status("sedov remesh_track_kernel")) return r;
    remesh_scan_kernel<<<1, 1024, 0, s>>>(M);
    if (int r = launch_status("sedov remesh_scan_kernel")) return r;
    remesh_pack_kernel<<<blocks, warps_per_block * 32, 0, s>>>(M);
    if (int r = launch_status("sedov remesh_pack_kernel")) return r;
    MARA_CUDA(cudaMemcpyAsync(cells_out, cell_offset_out + T, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    MARA_CUDA(cudaStreamSynchronize(s));
    return MARA_OK;
}

int mara_sedov_min_spacing(int32_t track_count, int64_t cells, const int64_t* cell_offset, const double* radii,
                           double* out, void* stream)
{
    MARA_REQUIRE(track_count >= 1 && cells >= 1 && cell_offset && radii && out, "mara_sedov_min_spacing: bad argument");
    cudaStream_t s = as_stream(stream);
    const double inf = INFINITY;
    MARA_CUDA(cudaMemcpyAsync(out, &inf, sizeof inf, cudaMemcpyHostToDevice, s));
    MARA_CUDA(cudaStreamSynchronize(s));   // the host value lives on this stack frame
    min_spacing_kernel<<<blocks_for(cells), 256, 0, s>>>(Tracks{track_count, cells, cell_offset, nullptr}, radii,
                                                         reinterpret_cast<unsigned long long*>(out));
    return launch_status("sedov min_spacing_kernel");
}

} // extern "C"
