// Constrained-transport ideal MHD on one periodic cube: the GB300 form of
// mara::advance_mhd_ct (src/scheme_mhd_v1.cpp:265-299, physics in
// src/physics_mhd.hpp:216-390, staggered operators in
// src/mesh_cartesian_3d.hpp:236-305) and the RK2 driver of
// examples/mhd3d.cpp:78-88,186-215.
//
// One stage = four kernels (FP64, or the mixed path with the fused stage off):
//   prim_kernel     face_to_cell + recover_primitive of every cell into P[N^3][8];
//                   fastest wavespeed reduced into the clock (CFL dt)
//   dt_kernel       dt = cfl * dl / max speed (scheme_mhd_v1.cpp:287)
//   face_kernel<a>  PLM slopes along axis a, face states, HLLE flux F[5] and the
//                   two transverse E-field components on all N+1 layers of the
//                   face array (layer N uses its own normal field bf[N], as the
//                   reference's flux_arrays does; cells are periodic)
//   update_kernel   (two launches: cells, then faces)
//                   u -= div(F) dt/dl; B.dA -= curl(E_edge) dt/dl, edge EMFs by
//                   the reference's face averaging (edge_emf_from_face);
//                   optionally averaged with the RK partner state.
// The mixed path on meshes with N a multiple of 32 replaces the face and
// update kernels by two fused launches (flux_kernel, emf_kernel, below) that
// also recover the next stage's primitives, with identical results.
// Layout: uc SoA [5][N][N][N] (any (component, cell) stride pair on input to
// the drop-in call); bf1 [N+1][N][N], bf2 [N][N+1][N], bf3 [N][N][N+1] as the
// reference holds them (the two periodic boundary layers stay identical).
//
// FP64: reference evaluation order. MIXED: P, F and E in FP32; u and B stay
// FP64 and are accumulated in FP64; the curl of the FP32 edge EMFs is formed
// from exact float-pair differences and rounded once to FP64, so div B is
// preserved to FP64 rounding as in the FP64 path. The mixed RK2 keeps stage
// 1's cell change as an FP32 increment (the minidisk's scheme), so that the
// cells of both stages take one FP64 addition per component per step; FP64
// runs at a small fraction of the FP32 rate on this part, and the update
// kernel was bound by its FP64 pipe.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include "common.cuh"
#include "mixed_math.cuh"
#include "mhd_physics.cuh"

namespace mara {
namespace mhd {

struct Clock
{
    double time;
    double dt[2];
    unsigned long long amax[2];   // fastest wavespeed bits (positive doubles order as integers)
    int64_t iteration;
    unsigned long long failures;  // zones with negative density or pressure
};

// Division by a divisor d fixed per launch, for numerators below 2^31
// (Granlund and Montgomery's round-up multiplier): q = (u m) >> s with
// s = 31 + ceil(log2 d) and m = ceil(2^s / d), exact because
// m d - 2^s < d <= 2^(s - 31). A 32-bit division by a runtime divisor takes
// some twenty integer instructions; this takes two.
struct FastDiv
{
    uint64_t m;
    uint32_t d;
    int s;
    __device__ uint32_t div(uint32_t u) const { return uint32_t((uint64_t(u) * m) >> s); }
};

inline FastDiv fast_div(uint32_t d)
{
    int l = 0;
    while ((uint64_t(1) << l) < d) ++l;
    FastDiv f;
    f.d = d;
    f.s = 31 + l;
    f.m = ((uint64_t(1) << f.s) + d - 1) / d;
    return f;
}

struct Args
{
    int N;
    FastDiv div_n, div_n1, div_nn, div_nn1;      // N, N + 1, N^2, N (N + 1)
    double gamma, dl, cfl, theta;
    const double* uc; int64_t ucs, uzs;          // input conserved, (component, cell) strides
    const double* bf[3];
    const double* uavg;                          // RK partner (SoA), or null
    const double* bavg[3];
    double* uc_out;                              // SoA
    double* bf_out[3];
    void* P;                                     // [N^3][8] cell records (double or float)
    void* F[3];                                  // [5][face count of axis a]
    void* E[3];                                  // [2][face count]: the two transverse components
    Clock* clock;
    int stage;
    float* dinc;                                 // [5][N^3] mixed RK2 stage-1 increments
    const double* next_uc;                       // fused mixed path: SoA state the next stage recovers from
};

// Cell updates of the mixed path (a template argument of the prim and update
// kernels): MIX_PLAIN writes u_out = u - du; MIX_INCREMENT (RK2 stage 1)
// writes only dinc = -du as floats; MIX_FROM_INCREMENT (stage 2) takes u0 from
// uc and u1 = u0 + dinc, and writes u_out = u0 + (dinc - du) / 2. Faces are
// updated in FP64 in every mode.
enum { MIX_PLAIN = 0, MIX_INCREMENT = 1, MIX_FROM_INCREMENT = 2 };

__host__ __device__ inline int64_t nb(int N, int axis) { return int64_t(N + (axis == 0)) * (N + (axis == 1)) * (N + (axis == 2)); }

__device__ inline int wrap(int i, int N) { return i < 0 ? i + N : (i >= N ? i - N : i); }

// element (i, j, k) of the face array of `axis`, (i, j, k) already in range
__device__ inline int64_t fidx(int N, int axis, int i, int j, int k)
{
    const int n1 = N + (axis == 1), n2 = N + (axis == 2);
    return (int64_t(i) * n1 + j) * n2 + k;
}

__device__ inline int64_t cidx(int N, int i, int j, int k) { return (int64_t(i) * N + j) * N + k; }

// 32-bit forms for the stage kernels: N <= 1024 is checked on the host, so
// every face array has fewer than 2^31 elements (component offsets stay 64-bit)
__device__ inline uint32_t nb32(int N, int axis)
{
    return uint32_t(N + (axis == 0)) * uint32_t(N + (axis == 1)) * uint32_t(N + (axis == 2));
}
__device__ inline uint32_t fidx32(int N, int axis, int i, int j, int k)
{
    const uint32_t n1 = N + (axis == 1), n2 = N + (axis == 2);
    return (uint32_t(i) * n1 + uint32_t(j)) * n2 + uint32_t(k);
}
__device__ inline uint32_t cidx32(int N, int i, int j, int k) { return (uint32_t(i) * N + uint32_t(j)) * N + uint32_t(k); }

// (i, j, k) of element u of the cell array (axis -1) or the face array of axis
__device__ inline void unflatten_fast(const Args& A, int axis, uint32_t u, int& i, int& j, int& k)
{
    const FastDiv& plane = axis < 1 ? A.div_nn : A.div_nn1;     // n1 n2: N^2 for cells and axis 0
    const FastDiv& row = axis == 2 ? A.div_n1 : A.div_n;        // n2
    const uint32_t a = plane.div(u), r = u - a * plane.d, b = row.div(r);
    i = int(a);
    j = int(b);
    k = int(r - b * row.d);
}

// (i, j, k) of linear index t of an n0 x n1 x n2 array, in 32-bit arithmetic
// (every array here has fewer than 2^31 elements: N <= 1024 is checked on the host)
__device__ inline void unflatten(int64_t t, int n1, int n2, int& i, int& j, int& k)
{
    const uint32_t u = uint32_t(t), plane = uint32_t(n1) * uint32_t(n2);
    const uint32_t a = u / plane, r = u - a * plane, b = r / uint32_t(n2);
    i = int(a);
    j = int(b);
    k = int(r - b * uint32_t(n2));
}

// The primitives of the stage kernels are one 8-value record per cell,
// [N^3][8] (rho, v, p, B), written and read as 16-byte vectors: a face reads
// its four stencil cells in 8 (FP32) or 16 (FP64) vector loads instead of 32
// scalar ones.
__device__ inline void store_cell(float* P, size_t c, const Prim<float>& p)
{
    float4* q = reinterpret_cast<float4*>(P + 8 * c);
    q[0] = make_float4(p.d, p.v[0], p.v[1], p.v[2]);
    q[1] = make_float4(p.p, p.b[0], p.b[1], p.b[2]);
}
__device__ inline void store_cell(double* P, size_t c, const Prim<double>& p)
{
    double2* q = reinterpret_cast<double2*>(P + 8 * c);
    q[0] = make_double2(p.d, p.v[0]);
    q[1] = make_double2(p.v[1], p.v[2]);
    q[2] = make_double2(p.p, p.b[0]);
    q[3] = make_double2(p.b[1], p.b[2]);
}
__device__ inline void load_cell(const float* P, size_t c, float out[8])
{
    const float4* q = reinterpret_cast<const float4*>(P + 8 * c);
    const float4 a = q[0], b = q[1];
    out[0] = a.x; out[1] = a.y; out[2] = a.z; out[3] = a.w;
    out[4] = b.x; out[5] = b.y; out[6] = b.z; out[7] = b.w;
}
__device__ inline void load_cell(const double* P, size_t c, double out[8])
{
    const double2* q = reinterpret_cast<const double2*>(P + 8 * c);
    for (int h = 0; h < 4; ++h)
    {
        const double2 v = q[h];
        out[2 * h] = v.x;
        out[2 * h + 1] = v.y;
    }
}

// The mixed recovery of cell c: face_to_cell in FP32 from the FP64 face
// fields, then recover_primitive (physics_mhd.hpp:290-303) in FP32 from the
// FP64 state (integer conversions, one reciprocal); only the energy
// difference E - kinetic - magnetic is taken in FP64. MIX_FROM_INCREMENT
// recovers u0 + the FP32 stage-1 increment. True where the reference throws
// (negative density or pressure). One function for the primitive kernel and
// the EMF kernel's next-stage recovery, so that both compile the same arithmetic.
struct Field3 { float b[3]; };
__device__ __forceinline__ Field3 cell_field(float x0, float x1, float y0, float y1, float z0, float z1)
{
    return Field3{{__fmul_rn(0.5f, __fadd_rn(x0, x1)), __fmul_rn(0.5f, __fadd_rn(y0, y1)),
                   __fmul_rn(0.5f, __fadd_rn(z0, z1))}};
}
// from the FP64 faces (each converted here; the EMF kernel converts each
// face once, when it updates it, and passes the floats)
__device__ __forceinline__ Field3 cell_field(double x0, double x1, double y0, double y1, double z0, double z1)
{
    return cell_field(d2f(x0), d2f(x1), d2f(y0), d2f(y1), d2f(z0), d2f(z1));
}

template<int MODE>
__device__ __forceinline__ bool recover_mixed(const double* uc, int64_t ucs, int64_t uzs, const float* dinc, int64_t NN,
                                              int64_t c, const Field3 f, float gm, Prim<float>& p)
{
    const double energy = uc[4 * ucs + c * uzs];
    p.d = d2f(uc[c * uzs]);
    float S[3] = {d2f(uc[ucs + c * uzs]), d2f(uc[2 * ucs + c * uzs]), d2f(uc[3 * ucs + c * uzs])};
    float de = 0.0f;   // energy increment, folded into the FP64 difference below
    if (MODE == MIX_FROM_INCREMENT)
    {
        p.d = __fadd_rn(p.d, dinc[c]);
        for (int q = 0; q < 3; ++q) S[q] = __fadd_rn(S[q], dinc[(q + 1) * NN + c]);
        de = dinc[4 * NN + c];
    }
    const float inv = rcp_fast(p.d);
    for (int q = 0; q < 3; ++q)
    {
        p.v[q] = div_corrected(S[q], p.d, inv);
        p.b[q] = f.b[q];
    }
    const float kin_mag = 0.5f * sum3(S, p.v) + 0.5f * sum3(f.b, f.b);
    p.p = d2f(energy - f2d(__fsub_rn(kin_mag, de))) * (gm - 1.0f);
    return p.d < 0.0f || p.p < 0.0f;
}

// ---------------------------------------------------------------- kernels
template<typename R, int MODE>
__global__ void __launch_bounds__(256, sizeof(R) == sizeof(float) ? 5 : 3) prim_kernel(const Args A)
{
    __shared__ double wmax[8];
    const int N = A.N;
    const int64_t NN = int64_t(N) * N * N;
    R* P = static_cast<R*>(A.P);
    const R gm = R(A.gamma);
    double m = 0.0;
    float mf = 0.0f;
    unsigned long long bad = 0;
    for (int64_t c = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; c < NN; c += int64_t(gridDim.x) * blockDim.x)
    {
        int i, j, k;
        unflatten_fast(A, -1, uint32_t(c), i, j, k);
        const uint32_t x0 = fidx32(N, 0, i, j, k), y0 = fidx32(N, 1, i, j, k), z0 = fidx32(N, 2, i, j, k);
        const uint32_t x1 = x0 + uint32_t(N) * N, y1 = y0 + N, z1 = z0 + 1;
        if constexpr (sizeof(R) == sizeof(float))
        {
            Prim<float> p;
            if (recover_mixed<MODE>(A.uc, A.ucs, A.uzs, A.dinc, NN, c,
                                    cell_field(A.bf[0][x0], A.bf[0][x1], A.bf[1][y0], A.bf[1][y1], A.bf[2][z0], A.bf[2][z1]),
                                    gm, p))
                ++bad;
            store_cell(P, c, p);
            mf = fmaxf(mf, fastest_speed(p, gm));
            continue;
        }
        const double b1 = 0.5 * (A.bf[0][x0] + A.bf[0][x1]);
        const double b2 = 0.5 * (A.bf[1][y0] + A.bf[1][y1]);
        const double b3 = 0.5 * (A.bf[2][z0] + A.bf[2][z1]);
        double u[5];
        for (int q = 0; q < 5; ++q) u[q] = A.uc[q * A.ucs + c * A.uzs];
        // recover_primitive (physics_mhd.hpp:290-303)
        const double d = u[0];
        const double S[3] = {u[1], u[2], u[3]}, b[3] = {b1, b2, b3};
        const double kin = 0.5 * sum3(S, S) / d;
        const double mag = 0.5 * sum3(b, b);
        const double pg = (u[4] - kin - mag) * (A.gamma - 1);
        Prim<R> p;
        p.d = R(d);
        for (int q = 0; q < 3; ++q)
        {
            p.v[q] = R(S[q] / d);
            p.b[q] = R(b[q]);
        }
        p.p = R(pg);
        if (d < 0.0 || pg < 0.0) ++bad;
        store_cell(P, c, p);
        m = fmax(m, double(fastest_speed(p, gm)));
    }
    if (sizeof(R) == sizeof(float)) m = double(mf);
    for (int o = 16; o > 0; o >>= 1)
    {
        m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        bad += __shfl_xor_sync(0xffffffffu, bad, o);
    }
    if ((threadIdx.x & 31) == 0)
    {
        wmax[threadIdx.x >> 5] = m;
        if (bad) atomicAdd(&A.clock->failures, bad);
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        double r = 0.0;
        for (int w = 0; w < int(blockDim.x >> 5); ++w) r = fmax(r, wmax[w]);
        atomicMax(&A.clock->amax[A.stage], (unsigned long long)__double_as_longlong(r));
    }
}

// begin: both stages' wavespeed maxima to zero. Otherwise dt of `stage`, and
// the other stage's maximum to zero (it was consumed by that stage's dt; the
// fused mixed path accumulates the next stage's maximum during this stage).
__global__ void dt_kernel(Clock* clock, int stage, double cfl, double dl, int begin)
{
    if (threadIdx.x != 0) return;
    if (begin) { clock->amax[0] = 0ull; clock->amax[1] = 0ull; }
    else
    {
        clock->dt[stage] = cfl * dl / __longlong_as_double((long long)clock->amax[stage]);
        clock->amax[stage ^ 1] = 0ull;
    }
}

// PLM face states from the four cells l-2 .. l+1 along AXIS (a, b | c, d)
// and the HLLE flux and transverse E-field of the face (godunov_fluxes_plm,
// scheme_mhd_v1.cpp:152-178). One function for the face kernels and the
// fused stage kernel, so that both compile the same arithmetic.
// The HLLE flux and E-field of a face from its two PLM states (the face's
// normal B is bl; the states' own normal components are not read).
template<typename R, int AXIS>
__device__ __forceinline__ void face_riemann(const R L[8], const R Rr[8], R bl, R gm, R F[5], R E[2])
{
    Prim<R> pl{L[0], {L[1], L[2], L[3]}, L[4], {L[5], L[6], L[7]}};
    Prim<R> pr{Rr[0], {Rr[1], Rr[2], Rr[3]}, Rr[4], {Rr[5], Rr[6], Rr[7]}};
    riemann_hlle<R, AXIS>(pl, pr, bl, gm, F, E);
}

template<typename R, int AXIS>
__device__ __forceinline__ void face_solve(const R xa[8], const R xb[8], const R xc[8], const R xd[8], R bl, R gm,
                                           R theta, R F[5], R E[2])
{
    R L[8], Rr[8];
    for (int q = 0; q < 8; ++q)
    {
        const R a = xa[q], b = xb[q], cc = xc[q], d = xd[q];
        if constexpr (sizeof(R) == sizeof(float))
        {
            // the doubled slope: the same face values in two multiplies fewer
            L[q] = __fmaf_rn(0.25f, plm2(a, b, cc, 2.0f * theta), b);
            Rr[q] = __fmaf_rn(-0.25f, plm2(b, cc, d, 2.0f * theta), cc);
        }
        else
        {
            L[q] = b + R(0.5) * plm(a, b, cc, theta);
            Rr[q] = cc - R(0.5) * plm(b, cc, d, theta);
        }
    }
    face_riemann<R, AXIS>(L, Rr, bl, gm, F, E);
}

template<typename R, int AXIS>
__global__ void face_kernel(const Args A)
{
    const int N = A.N;
    const uint32_t NF = nb32(N, AXIS);
    const R* P = static_cast<const R*>(A.P);
    R* F = static_cast<R*>(A.F[AXIS]);
    R* E = static_cast<R*>(A.E[AXIS]);
    const R gm = R(A.gamma), theta = R(A.theta);
    // the stencil's cells l-2 .. l+1 lie on the line along AXIS through the
    // face: a base index (AXIS coordinate zero) plus the wrapped layer x stride
    const uint32_t stride = AXIS == 0 ? uint32_t(N) * N : (AXIS == 1 ? uint32_t(N) : 1u);
    for (uint32_t f = blockIdx.x * blockDim.x + threadIdx.x; f < NF; f += gridDim.x * blockDim.x)
    {
        int i, j, k;
        unflatten_fast(A, AXIS, f, i, j, k);
        const int l = AXIS == 0 ? i : (AXIS == 1 ? j : k);
        const uint32_t base = cidx32(N, AXIS == 0 ? 0 : i, AXIS == 1 ? 0 : j, AXIS == 2 ? 0 : k);
        const uint32_t cm2 = base + uint32_t(wrap(l - 2, N)) * stride, cm1 = base + uint32_t(wrap(l - 1, N)) * stride;
        const uint32_t c0 = base + uint32_t(wrap(l, N)) * stride, cp1 = base + uint32_t(wrap(l + 1, N)) * stride;
        R xa[8], xb[8], xc[8], xd[8];
        load_cell(P, cm2, xa);
        load_cell(P, cm1, xb);
        load_cell(P, c0, xc);
        load_cell(P, cp1, xd);
        R fl[5], e[2];
        face_solve<R, AXIS>(xa, xb, xc, xd, R(A.bf[AXIS][f]), gm, theta, fl, e);
        for (int q = 0; q < 5; ++q) F[q * size_t(NF) + f] = fl[q];
        E[f] = e[0];
        E[size_t(NF) + f] = e[1];
    }
}

// E component `comp` on the faces of `axis`: layer index along `axis` taken
// as is (0..N), transverse cell indices periodic. Face E arrays hold the two
// transverse components in increasing axis order; nbv[a] is the size of the
// face array of axis a.
template<typename T>
__device__ inline T ef_raw(const Args& A, const uint32_t nbv[3], int axis, int comp, int i, int j, int k)
{
    const int N = A.N;
    if (axis != 0) i = wrap(i, N);
    if (axis != 1) j = wrap(j, N);
    if (axis != 2) k = wrap(k, N);
    const size_t slot = comp < axis ? comp : comp - 1;
    return static_cast<const T*>(A.E[axis])[slot * nbv[axis] + fidx32(N, axis, i, j, k)];
}

template<typename R>
__device__ inline double ef(const Args& A, const uint32_t nbv[3], int axis, int comp, int i, int j, int k)
{
    return double(ef_raw<R>(A, nbv, axis, comp, i, j, k));
}

// edge_emf_from_face (scheme_mhd_v1.cpp:76-98); edge of axis a at (i, j, k)
// starts at corner (i, j, k). Averages in the reference's order.
template<typename R>
__device__ inline double ee(const Args& A, const uint32_t nbv[3], int axis, int i, int j, int k)
{
    // explicit rounding: every face sharing the edge must see the same double
    auto avg = [](double x, double y) { return __dmul_rn(0.5, __dadd_rn(x, y)); };
    double a, b;
    if (axis == 0)
    {
        a = avg(ef<R>(A, nbv, 1, 0, i, j, k - 1), ef<R>(A, nbv, 1, 0, i, j, k));
        b = avg(ef<R>(A, nbv, 2, 0, i, j - 1, k), ef<R>(A, nbv, 2, 0, i, j, k));
    }
    else if (axis == 1)
    {
        a = avg(ef<R>(A, nbv, 2, 1, i - 1, j, k), ef<R>(A, nbv, 2, 1, i, j, k));
        b = avg(ef<R>(A, nbv, 0, 1, i, j, k - 1), ef<R>(A, nbv, 0, 1, i, j, k));
    }
    else
    {
        a = avg(ef<R>(A, nbv, 0, 2, i, j - 1, k), ef<R>(A, nbv, 0, 2, i, j, k));
        b = avg(ef<R>(A, nbv, 1, 2, i - 1, j, k), ef<R>(A, nbv, 1, 2, i, j, k));
    }
    return avg(a, b);
}

// The mixed form of ee: the same averages in FP32, every operation rounded
// explicitly (no contraction), so each edge EMF is one fixed function of the
// four face values around it and every face that shares the edge sees the
// same float; differences of floats are exact in FP64.
__device__ inline float ee_f(const Args& A, const uint32_t nbv[3], int axis, int i, int j, int k)
{
    auto e = [&](int ax, int comp, int a, int b, int c) { return ef_raw<float>(A, nbv, ax, comp, a, b, c); };
    auto avg = [](float x, float y) { return __fmul_rn(0.5f, __fadd_rn(x, y)); };
    float a, b;
    if (axis == 0)
    {
        a = avg(e(1, 0, i, j, k - 1), e(1, 0, i, j, k));
        b = avg(e(2, 0, i, j - 1, k), e(2, 0, i, j, k));
    }
    else if (axis == 1)
    {
        a = avg(e(2, 1, i - 1, j, k), e(2, 1, i, j, k));
        b = avg(e(0, 1, i, j, k - 1), e(0, 1, i, j, k));
    }
    else
    {
        a = avg(e(0, 2, i, j - 1, k), e(0, 2, i, j, k));
        b = avg(e(1, 2, i - 1, j, k), e(1, 2, i, j, k));
    }
    return avg(a, b);
}

// a - b as the unrounded pair s + e of floats (Knuth's TwoSum, 6 operations,
// each rounded explicitly so the compiler can neither contract nor reorder)
__device__ inline void two_diff(float a, float b, float& s, float& e)
{
    s = __fsub_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(-b, bb));
}

// (a - b) - (c - d) of four floats, as a double: the three differences are
// exact float pairs; only the sum of the three rounding terms rounds (in
// FP32, at 2^-24 of the terms, themselves at most half an ulp of a - b and
// c - d), then hi + lo is one FP64 addition. Equal to the FP64 curl of the
// float EMFs up to rounding far below the FP64 rounding of the face update.
__device__ inline double curl_f(float a, float b, float c, float d)
{
    float s1, e1, s2, e2, s3, e3;
    two_diff(a, b, s1, e1);
    two_diff(c, d, s2, e2);
    two_diff(s1, s2, s3, e3);
    return f2d(s3) + f2d(__fadd_rn(__fsub_rn(e1, e2), e3));
}

// x / 2 by decrementing the exponent: exact, and equal to x * 0.5, for every
// normal x above the smallest normal double times 2; zero, subnormals, the
// two smallest binades, infinities and NaN are returned unchanged (an error
// below 4.5e-308 for the tiny ones). Integer instructions only.
__device__ inline double half_exact(double x)
{
    const long long b = __double_as_longlong(x);
    const unsigned e = unsigned(b >> 52) & 0x7FFu;
    return e >= 2u && e <= 0x7FEu ? __longlong_as_double(b - (1LL << 52)) : x;
}

// PART 0: the cells (MODE applies); PART 1: the three face arrays (FP64 in
// every mode). Two launches, so that each part gets its own register budget:
// both wait on scattered reads, and the face part at 32 registers runs eight
// blocks per SM (the single kernel ran five; measured 0.704 -> 0.661 ms per
// 128^3 step).
template<typename R, int MODE, int PART>
__global__ void __launch_bounds__(256, sizeof(R) == sizeof(float) ? (PART == 0 ? 5 : 8) : 4)
update_kernel(const Args A)
{
    const int N = A.N;
    const int64_t NN = int64_t(N) * N * N;
    const double dt = A.clock->dt[A.stage];
    const double dl = A.dl;
    // dt / dl once per block: an FP64 division and conversion per thread
    // would cost more FP64-pipe issue than the update itself
    __shared__ double s_dtdl;
    __shared__ float s_dtdl_f;
    if (threadIdx.x == 0)
    {
        s_dtdl = dt / dl;
        s_dtdl_f = float(s_dtdl);
    }
    __syncthreads();
    const double dt_over_dl_d = s_dtdl;
    const float dt_over_dl = s_dtdl_f;
    const uint32_t nbv[3] = {nb32(N, 0), nb32(N, 1), nb32(N, 2)};
    const int64_t nf0 = nbv[0], nf1 = nbv[1], nf2 = nbv[2];
    const int64_t begin = PART == 0 ? 0 : NN, end = PART == 0 ? NN : NN + nf0 + nf1 + nf2;
    for (int64_t t = begin + blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < end; t += int64_t(gridDim.x) * blockDim.x)
    {
        if (PART == 0)
        {
            const int64_t c = t;
            int i, j, k;
            unflatten_fast(A, -1, uint32_t(c), i, j, k);
            const uint32_t x0 = fidx32(N, 0, i, j, k), x1 = x0 + uint32_t(N) * N;
            const uint32_t y0 = fidx32(N, 1, i, j, k), y1 = y0 + N;
            const uint32_t z0 = fidx32(N, 2, i, j, k), z1 = z0 + 1;
            for (int q = 0; q < 5; ++q)
            {
                const R* F0 = static_cast<const R*>(A.F[0]) + q * nf0;
                const R* F1 = static_cast<const R*>(A.F[1]) + q * nf1;
                const R* F2 = static_cast<const R*>(A.F[2]) + q * nf2;
                double out;
                if (sizeof(R) == sizeof(double))
                {
                    const double u = A.uc[q * A.ucs + c * A.uzs];
                    const double dc = (double(F0[x1]) - double(F0[x0])) + (double(F1[y1]) - double(F1[y0]))
                                    + (double(F2[z1]) - double(F2[z0]));
                    out = u - dc * dt / dl;
                }
                else
                {
                    const float dc = (float(F0[x1]) - float(F0[x0])) + (float(F1[y1]) - float(F1[y0]))
                                   + (float(F2[z1]) - float(F2[z0]));
                    const float du = __fmul_rn(dc, dt_over_dl);
                    if (MODE == MIX_INCREMENT)
                    {
                        A.dinc[q * NN + c] = -du;
                        continue;
                    }
                    const double u = A.uc[q * A.ucs + c * A.uzs];
                    if (MODE == MIX_FROM_INCREMENT)
                        out = u + f2d_sum(__fmul_rn(0.5f, __fsub_rn(A.dinc[q * NN + c], du)));
                    else
                        out = u - f2d_sum(du);
                }
                // weighted_sum a*0.5 + b*(1-0.5): halving is exact, so (a + b)*0.5 is the same double
                if (A.uavg) out = sizeof(R) == sizeof(float) ? half_exact(A.uavg[q * NN + c] + out)
                                                             : A.uavg[q * NN + c] * 0.5 + out * (1 - 0.5);
                A.uc_out[q * NN + c] = out;
            }
            continue;
        }
        int64_t f = t - NN;
        int axis = 0;
        if (f >= nf0) { f -= nf0; axis = 1; if (f >= nf1) { f -= nf1; axis = 2; } }
        int i, j, k;
        unflatten_fast(A, axis, uint32_t(f), i, j, k);
        // solenoidal_difference (mesh_cartesian_3d.hpp:265-274)
        if constexpr (sizeof(R) == sizeof(float))
        {
            double cf;
            if (axis == 0)
                cf = curl_f(ee_f(A, nbv, 2, i, j + 1, k), ee_f(A, nbv, 2, i, j, k), ee_f(A, nbv, 1, i, j, k + 1), ee_f(A, nbv, 1, i, j, k));
            else if (axis == 1)
                cf = curl_f(ee_f(A, nbv, 0, i, j, k + 1), ee_f(A, nbv, 0, i, j, k), ee_f(A, nbv, 2, i + 1, j, k), ee_f(A, nbv, 2, i, j, k));
            else
                cf = curl_f(ee_f(A, nbv, 1, i + 1, j, k), ee_f(A, nbv, 1, i, j, k), ee_f(A, nbv, 0, i, j + 1, k), ee_f(A, nbv, 0, i, j, k));
            double out = fma(-cf, dt_over_dl_d, A.bf[axis][f]);
            if (A.bavg[axis]) out = half_exact(A.bavg[axis][f] + out);
            A.bf_out[axis][f] = out;
            continue;
        }
        double cf;
        if (axis == 0)
            cf = (ee<R>(A, nbv, 2, i, j + 1, k) - ee<R>(A, nbv, 2, i, j, k)) - (ee<R>(A, nbv, 1, i, j, k + 1) - ee<R>(A, nbv, 1, i, j, k));
        else if (axis == 1)
            cf = (ee<R>(A, nbv, 0, i, j, k + 1) - ee<R>(A, nbv, 0, i, j, k)) - (ee<R>(A, nbv, 2, i + 1, j, k) - ee<R>(A, nbv, 2, i, j, k));
        else
            cf = (ee<R>(A, nbv, 1, i + 1, j, k) - ee<R>(A, nbv, 1, i, j, k)) - (ee<R>(A, nbv, 0, i, j + 1, k) - ee<R>(A, nbv, 0, i, j, k));
        double out = A.bf[axis][f] - cf * dt / dl;
        if (A.bavg[axis]) out = A.bavg[axis][f] * 0.5 + out * (1 - 0.5);
        A.bf_out[axis][f] = out;
    }
}

// ---------------------------------------------------------------- fused mixed stage
// The mixed stage as two launches in place of the three face kernels and the
// two update launches, with the same arithmetic (the results are identical).
// Both own a TJ x TK column of cells (j, k) per block and march along i over
// a chunk [i0, i1) of cell planes.
//
// flux_kernel: per plane c, the x faces of layer c+1 and the y and z faces of
// plane c (each tile solves its own faces and those of the high neighbour
// row / column that its cells need: no face is solved by more than two
// tiles), then the cells of plane c from the fluxes held in shared memory.
// The face E-fields go to global memory (F never does).
//
// emf_kernel: per plane c, the face E-fields of layer c and planes c-1, c
// (with a one-face halo) into shared memory, the edge EMFs at i = c, then the
// x faces of layer c and the y and z faces of plane c-1 (they need the EMFs of
// the plane above, so they trail by one plane), and then, optionally, the
// primitives of the next RK stage for the cells of plane c-1 from the
// updated state and faces, with the next stage's fastest wavespeed: the
// primitive kernel runs only for the first stage of a call.
namespace fused {
constexpr int TJ = 8, TK = 32;
// Threads per block. Nine warps let a plane's 832 face updates (EMF) take
// three rounds per thread instead of a fourth for a quarter of the threads;
// for the 808 face solves (flux) nine warps held the kernel to 56 registers
// and were slower. Measured at 128^3 (RK2 step, flux/EMF threads):
// 256/256 0.502 ms, 288/288 0.505, 288/256 0.509, 256/288 0.497.
constexpr int FLUX_THREADS = 256, EMF_THREADS = 288;
// Face E-fields in the EMF kernel, rows of XK (YK, ZK) floats with element
// kk at row offset kk + 4 (kk + 1 for z), so that the x and y rows' interior
// kk in [0, TK) is 16-byte aligned for vector copies
constexpr int XK = TK + 8, XN = (TJ + 2) * XK;      // x-face E: jj in [-1, TJ], kk in [-1, TK]
constexpr int YK = TK + 8, YN = (TJ + 1) * YK;      // y-face E: jj in [0, TJ], kk in [-1, TK]
constexpr int ZK = TK + 4, ZN = (TJ + 2) * ZK;      // z-face E: jj in [-1, TJ], kk in [0, TK] (rows padded to 16 B)
constexpr int XO = 4, YO = 4;                       // row offset of kk = 0
constexpr int FXN = TJ * TK;                        // x faces of the tile
constexpr int FYN = (TJ + 1) * TK;                  // y faces: jj in [0, TJ], kk in [0, TK)
constexpr int FZK = TK + 1, FZN = TJ * FZK;         // z faces: jj in [0, TJ), kk in [0, TK]
constexpr int E0K = TK + 1, E0N = (TJ + 1) * E0K;   // EMFs along i: jj in [0, TJ], kk in [0, TK]
constexpr int E1K = TK + 1, E1N = TJ * E1K;         // along j: jj in [0, TJ), kk in [0, TK]
constexpr int E2K = TK, E2N = (TJ + 1) * E2K;       // along k: jj in [0, TJ], kk in [0, TK)
constexpr int pad32(int n) { return (n + 31) & ~31; }
// the flux kernel's face items per plane, each kind padded to whole warps so
// that no warp mixes kinds
constexpr int SOLVE_Y = pad32(FYN), SOLVE_Z = pad32(FZN);
// copies per plane: x and y rows as TK/4 16-byte pieces plus the two halo
// elements; z rows (N + 1 floats, unaligned) element by element
constexpr int ROW_PIECES = TK / 4 + 2;
// z rows: TK/4 16-byte pieces (kk in [0, TK)) plus the element kk = TK, from
// the fused path's padded z-face E layout (zrow_e below)
constexpr int ZROW_PIECES = TK / 4 + 1;
constexpr int LOAD_X = 2 * (TJ + 2) * ROW_PIECES, LOAD_Y = 2 * (TJ + 1) * ROW_PIECES, LOAD_Z = 2 * (TJ + 2) * ZROW_PIECES;

struct __align__(16) FluxSmem
{
    float xl[8][FXN];          // the next x layer's left states (cell c+1's high-side PLM values), per thread
    double uc[5][FXN];         // the cells' state of plane c (staged during the solves)
    float dinc[5][FXN];        // their FP32 stage-1 increments (RK2 stage 2)
    float fx[2][5][FXN];       // x-face fluxes; layer l in slot l & 1
    float fy[5][FYN];          // y-face fluxes of plane c
    float fz[5][FZN];
};

struct __align__(16) EmfSmem
{
    float ex[2][2][XN];        // x-face E components 1, 2; layer l in slot l & 1
    float ey[3][2][YN];        // y-face E components 0, 2; plane p in slot p mod 3
    float ez[3][2][ZN];        // z-face E components 0, 1
    double bin[FXN + FYN + FZN];   // the faces' input field (staged during the edge phase):
    double bav[FXN + FYN + FZN];   // x faces of the tile, y rows [0, TJ], z columns [0, TK]; the RK partner
    float e0[2][E0N], e1[2][E1N], e2[2][E2N];
    double bx[2][FXN];         // updated x faces; layer l in slot l & 1
    double by[FYN];            // updated y faces of plane c-1 (row TJ: the neighbour's, for the cells)
    double bz[FZN];
    float bxf[2][FXN], byf[FYN], bzf[FZN];   // their FP32 images for the next-stage recovery (NEXT)
    double wmax[EMF_THREADS / 32];
    unsigned long long wbad[EMF_THREADS / 32];
};

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem)
{
    const unsigned s = unsigned(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem)
{
    const unsigned s = unsigned(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_prior() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ int mod3(int p) { return (p % 3 + 3) % 3; }
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem)
{
    const unsigned s = unsigned(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

__device__ __forceinline__ float avg(float x, float y) { return __fmul_rn(0.5f, __fadd_rn(x, y)); }

// The fused path's z-face E-fields: rows of N + 4 floats (N + 1 faces,
// padded so that every row starts on 16 bytes and the EMF kernel copies it
// in 16-byte pieces); the face (i, j, k) and the component stride.
__device__ __forceinline__ uint32_t zrow_e(int N, int i, int j, int k)
{
    return (uint32_t(i) * uint32_t(N) + uint32_t(j)) * uint32_t(N + 4) + uint32_t(k);
}
__device__ __forceinline__ uint32_t zrow_nb(int N) { return uint32_t(N) * uint32_t(N) * uint32_t(N + 4); }

struct Tile
{
    int j0, k0, i0, i1;
    bool last_j, last_k;
};

__device__ __forceinline__ Tile tile_of(int N, int chunks)
{
    const int tiles_k = N / TK, tiles = (N / TJ) * tiles_k;
    const int chunk = int(blockIdx.x) / tiles, tile = int(blockIdx.x) - chunk * tiles;
    Tile t;
    t.j0 = (tile / tiles_k) * TJ;
    t.k0 = (tile % tiles_k) * TK;
    t.i0 = int(int64_t(chunk) * N / chunks);
    t.i1 = int(int64_t(chunk + 1) * N / chunks);
    t.last_j = t.j0 + TJ == N;
    t.last_k = t.k0 + TK == N;
    return t;
}
} // namespace fused

// The four primitive records of a face stencil, read from global memory (the
// primitive array is small enough to stay in L2).
__device__ __forceinline__ void stencil(const float* P, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, float xa[8],
                                        float xb[8], float xc[8], float xd[8])
{
    load_cell(P, c0, xa);
    load_cell(P, c1, xb);
    load_cell(P, c2, xc);
    load_cell(P, c3, xd);
}

template<int MODE>
__global__ void __launch_bounds__(fused::FLUX_THREADS, 4) flux_kernel(const Args A, int chunks)
{
    using namespace fused;
    __shared__ FluxSmem S;
    __shared__ float s_dtdl;
    const int N = A.N;
    const Tile T = tile_of(N, chunks);
    const float* P = static_cast<const float*>(A.P);
    const float gm = float(A.gamma), theta = float(A.theta);
    const int64_t NN = int64_t(N) * N * N;
    const uint32_t nbv[3] = {nb32(N, 0), nb32(N, 1), nb32(N, 2)};
    float* E0 = static_cast<float*>(A.E[0]);
    float* E1 = static_cast<float*>(A.E[1]);
    float* E2 = static_cast<float*>(A.E[2]);
    if (threadIdx.x == 0) s_dtdl = float(A.clock->dt[A.stage] / A.dl);

    // x faces of layer lx over the tile: fluxes into slot lx & 1, E-fields
    // out when this chunk owns the layer. Thread t always takes the x face
    // column t (FLUX_THREADS == FXN), so the left state of layer lx (cell
    // lx-1's high side) is the one this thread formed at layer lx-1 from the
    // same slope as that layer's right state, kept in S.xl; only the chunk's
    // first layer computes it. The same floats as face_solve.
    static_assert(FLUX_THREADS == FXN, "one x face column per thread");
    auto solve_x = [&](int t, int lx, bool write_e, bool first) {
        const int jj = t / TK, kk = t - jj * TK;
        const int j = T.j0 + jj, k = T.k0 + kk;
        float xb[8], xc[8], xd[8], L[8], Rr[8], F[5], Ef[2];
        load_cell(P, cidx32(N, wrap(lx - 1, N), j, k), xb);
        load_cell(P, cidx32(N, wrap(lx, N), j, k), xc);
        load_cell(P, cidx32(N, wrap(lx + 1, N), j, k), xd);
        if (first)
        {
            float xa[8];
            load_cell(P, cidx32(N, wrap(lx - 2, N), j, k), xa);
            for (int q = 0; q < 8; ++q) L[q] = __fmaf_rn(0.25f, plm2(xa[q], xb[q], xc[q], 2.0f * theta), xb[q]);
        }
        else
            for (int q = 0; q < 8; ++q) L[q] = q == 5 ? 0.0f : S.xl[q][t];    // component 5: the normal B, not read
        for (int q = 0; q < 8; ++q)
        {
            if (q == 5)
            {
                Rr[q] = 0.0f;
                continue;
            }
            const float g = plm2(xb[q], xc[q], xd[q], 2.0f * theta);
            Rr[q] = __fmaf_rn(-0.25f, g, xc[q]);
            S.xl[q][t] = __fmaf_rn(0.25f, g, xc[q]);
        }
        const uint32_t f = fidx32(N, 0, lx, j, k);
        face_riemann<float, 0>(L, Rr, float(A.bf[0][f]), gm, F, Ef);
        for (int n = 0; n < 5; ++n) S.fx[lx & 1][n][t] = F[n];
        if (write_e)
        {
            E0[f] = Ef[0];
            E0[size_t(nbv[0]) + f] = Ef[1];
        }
    };

    // the cell update's inputs go through shared memory, copied while the
    // faces are solved: SoA state (component stride a multiple of two
    // doubles, 16-byte aligned) and the FP32 increments
    constexpr bool READS_U = MODE != MIX_INCREMENT, READS_D = MODE == MIX_FROM_INCREMENT;
    const bool stage_u = READS_U && A.uzs == 1 && A.ucs % 2 == 0 && (reinterpret_cast<uintptr_t>(A.uc) & 15) == 0;
    auto stage_cells = [&](int c) {
        // rows of TK cells: TK/2 16-byte pieces of state, TK/4 of increments, per component
        // (every division below is by a power-of-two constant: a shift)
        constexpr int UP = TJ * TK / 2, DP = TJ * TK / 4;
        static_assert((UP & (UP - 1)) == 0 && (DP & (DP - 1)) == 0 && (TK & (TK - 1)) == 0, "shift decoding");
        for (int t = threadIdx.x; t < 5 * (UP + DP); t += FLUX_THREADS)
        {
            if (t < 5 * UP)
            {
                const int q = t / UP, w = t - q * UP, jj = w / (TK / 2), piece = w - jj * (TK / 2);
                const int64_t cell = cidx32(N, c, T.j0 + jj, T.k0);
                if (stage_u) cp_async16(&S.uc[q][jj * TK + 2 * piece], A.uc + q * A.ucs + cell + 2 * piece);
            }
            else if (READS_D)
            {
                const int v = t - 5 * UP, q = v / DP, w = v - q * DP, jj = w / (TK / 4), piece = w - jj * (TK / 4);
                const int64_t cell = cidx32(N, c, T.j0 + jj, T.k0);
                cp_async16(&S.dinc[q][jj * TK + 4 * piece], A.dinc + q * NN + cell + 4 * piece);
            }
        }
        cp_async_commit();
    };

    solve_x(threadIdx.x, T.i0, true, true);
    for (int c = T.i0; c < T.i1; ++c)
    {
        __syncthreads();                   // the previous plane's cell updates are done
        if (READS_U) stage_cells(c);
        const bool x_owned = c + 1 < T.i1 || c + 1 == N;
        for (int t = threadIdx.x; t < FXN + SOLVE_Y + SOLVE_Z; t += FLUX_THREADS)
        {
            if (t < FXN)
            {
                solve_x(t, c + 1, x_owned, false);
            }
            else if (t < FXN + SOLVE_Y)
            {
                const int u = t - FXN;
                if (u >= FYN) continue;
                const int jj = u / TK, kk = u - jj * TK;            // jj = TJ: the high neighbour's face
                const int j = T.j0 + jj, k = T.k0 + kk;
                float xa[8], xb[8], xc[8], xd[8], F[5], Ef[2];
                stencil(P, cidx32(N, c, wrap(j - 2, N), k), cidx32(N, c, wrap(j - 1, N), k), cidx32(N, c, wrap(j, N), k),
                        cidx32(N, c, wrap(j + 1, N), k), xa, xb, xc, xd);
                const uint32_t f = fidx32(N, 1, c, j, k);
                face_solve<float, 1>(xa, xb, xc, xd, float(A.bf[1][f]), gm, theta, F, Ef);
                for (int n = 0; n < 5; ++n) S.fy[n][u] = F[n];
                if (jj < TJ || T.last_j)
                {
                    E1[f] = Ef[0];
                    E1[size_t(nbv[1]) + f] = Ef[1];
                }
            }
            else
            {
                const int u = t - FXN - SOLVE_Y;
                if (u >= FZN) continue;
                const int jj = u / FZK, kk = u - jj * FZK;           // kk = TK: the high neighbour's face
                const int j = T.j0 + jj, k = T.k0 + kk;
                float xa[8], xb[8], xc[8], xd[8], F[5], Ef[2];
                stencil(P, cidx32(N, c, j, wrap(k - 2, N)), cidx32(N, c, j, wrap(k - 1, N)), cidx32(N, c, j, wrap(k, N)),
                        cidx32(N, c, j, wrap(k + 1, N)), xa, xb, xc, xd);
                const uint32_t f = fidx32(N, 2, c, j, k);
                face_solve<float, 2>(xa, xb, xc, xd, float(A.bf[2][f]), gm, theta, F, Ef);
                for (int n = 0; n < 5; ++n) S.fz[n][u] = F[n];
                if (kk < TK || T.last_k)
                {
                    const uint32_t fe = zrow_e(N, c, j, k);
                    E2[fe] = Ef[0];
                    E2[size_t(zrow_nb(N)) + fe] = Ef[1];
                }
            }
        }
        if (READS_U) cp_async_wait_all();
        __syncthreads();
        const float dtdl = s_dtdl;
        for (int t = threadIdx.x; t < FXN; t += FLUX_THREADS)
        {
            const int jj = t / TK, kk = t - jj * TK;
            const int64_t cell = cidx32(N, c, T.j0 + jj, T.k0 + kk);
            for (int q = 0; q < 5; ++q)
            {
                const float* fy = S.fy[q];
                const float* fz = S.fz[q];
                const float dc = (S.fx[(c + 1) & 1][q][t] - S.fx[c & 1][q][t]) + (fy[(jj + 1) * TK + kk] - fy[jj * TK + kk])
                               + (fz[jj * FZK + kk + 1] - fz[jj * FZK + kk]);
                const float du = __fmul_rn(dc, dtdl);
                if (MODE == MIX_INCREMENT)
                {
                    A.dinc[q * NN + cell] = -du;
                    continue;
                }
                const double u = stage_u ? S.uc[q][t] : A.uc[q * A.ucs + cell * A.uzs];
                double out = MODE == MIX_FROM_INCREMENT ? u + f2d_sum(__fmul_rn(0.5f, __fsub_rn(S.dinc[q][t], du)))
                                                        : u - f2d_sum(du);
                if (A.uavg) out = half_exact(A.uavg[q * NN + cell] + out);
                A.uc_out[q * NN + cell] = out;
            }
        }
    }
}

// NEXT: the primitives the EMF kernel recovers for the next RK stage:
// 0 none, MIX_INCREMENT (the next step's first stage: from A.next_uc) or
// MIX_FROM_INCREMENT (the second stage: A.next_uc plus the FP32 increment).
template<int NEXT>
__global__ void __launch_bounds__(fused::EMF_THREADS, 4) emf_kernel(const Args A, int chunks)
{
    using namespace fused;
    extern __shared__ __align__(16) unsigned char emf_smem[];
    EmfSmem& S = *reinterpret_cast<EmfSmem*>(emf_smem);
    __shared__ double s_dtdl;
    const int N = A.N;
    const Tile T = tile_of(N, chunks);
    const uint32_t nbv[3] = {nb32(N, 0), nb32(N, 1), nb32(N, 2)};
    const float* E0 = static_cast<const float*>(A.E[0]);
    const float* E1 = static_cast<const float*>(A.E[1]);
    const float* E2 = static_cast<const float*>(A.E[2]);
    const int64_t NN = int64_t(N) * N * N;
    const float gm = float(A.gamma);
    if (threadIdx.x == 0) s_dtdl = A.clock->dt[A.stage] / A.dl;

    // face E-fields of layer lx (when load_x) and of plane py, as one cp.async group
    auto load = [&](bool load_x, int lx, int py) {
        const uint32_t pw = uint32_t(wrap(py, N));
        for (int t = threadIdx.x; t < LOAD_X + LOAD_Y + LOAD_Z; t += EMF_THREADS)
        {
            if (t < LOAD_X + LOAD_Y)
            {
                // row piece: 0 .. TK/4-1 the interior, TK/4 kk = -1, TK/4+1 kk = TK
                const bool x = t < LOAD_X;
                if (x && !load_x) continue;
                const int v = x ? t : t - LOAD_X;
                const int row = v / ROW_PIECES, piece = v - row * ROW_PIECES;
                // two components of `rows` rows each: the component is a
                // comparison, not a division by a runtime row count
                const int rows = x ? TJ + 2 : TJ + 1, h = row >= rows ? 1 : 0, r = row - h * rows;
                const int kk = piece < TK / 4 ? 4 * piece : (piece == TK / 4 ? -1 : TK);
                const uint32_t f = x ? fidx32(N, 0, lx, wrap(T.j0 + r - 1, N), wrap(T.k0 + kk, N))
                                     : fidx32(N, 1, pw, T.j0 + r, wrap(T.k0 + kk, N));
                const float* src = x ? E0 + size_t(h) * nbv[0] + f : E1 + size_t(h) * nbv[1] + f;
                float* dst = x ? &S.ex[lx & 1][h][r * XK + XO + kk] : &S.ey[mod3(py)][h][r * YK + YO + kk];
                if (piece < TK / 4) cp_async16(dst, src);
                else cp_async4(dst, src);
            }
            else
            {
                const int v = t - LOAD_X - LOAD_Y, h = v >= LOAD_Z / 2 ? 1 : 0, u = v - h * (LOAD_Z / 2);
                const int r = u / ZROW_PIECES, piece = u - r * ZROW_PIECES;   // jj = r - 1
                const int kk = piece < TK / 4 ? 4 * piece : TK;
                const float* src = E2 + size_t(h) * zrow_nb(N) + zrow_e(N, pw, wrap(T.j0 + r - 1, N), T.k0 + kk);
                float* dst = &S.ez[mod3(py)][h][r * ZK + kk];
                if (piece < TK / 4) cp_async16(dst, src);
                else cp_async4(dst, src);
            }
        }
        cp_async_commit();
    };

    // the face update's inputs of step c (x faces of layer c; y and z faces
    // of plane c-1 unless `first`), as one cp.async group: x and y rows in
    // 16-byte pieces (rows of TK doubles start at multiples of 32 elements),
    // z rows (N + 1 doubles) element by element
    const bool with_avg = A.bavg[0] != nullptr;
    auto aligned16 = [](const void* q) { return (reinterpret_cast<uintptr_t>(q) & 15) == 0; };
    const bool vec = aligned16(A.bf[0]) && aligned16(A.bf[1]) && (!with_avg || (aligned16(A.bavg[0]) && aligned16(A.bavg[1])));
    auto piece16 = [&](double* dst, const double* src) {
        if (vec) cp_async16(dst, src);
        else
        {
            cp_async8(dst, src);
            cp_async8(dst + 1, src + 1);
        }
    };
    auto stage_faces = [&](int c, bool first) {
        constexpr int XP = TJ * TK / 2, YP = (TJ + 1) * TK / 2;
        const int arrays = with_avg ? 2 : 1;
        for (int t = threadIdx.x; t < arrays * (XP + YP + FZN); t += EMF_THREADS)
        {
            const int a = t >= XP + YP + FZN ? 1 : 0, v = t - a * (XP + YP + FZN);
            double* dst = a ? S.bav : S.bin;
            const double* const* src = a ? A.bavg : A.bf;
            if (v < XP)
            {
                const int jj = v / (TK / 2), piece = v - jj * (TK / 2);
                piece16(dst + jj * TK + 2 * piece, src[0] + fidx32(N, 0, c, T.j0 + jj, T.k0 + 2 * piece));
            }
            else if (v < XP + YP)
            {
                if (first) continue;
                const int w = v - XP, jj = w / (TK / 2), piece = w - jj * (TK / 2);
                piece16(dst + FXN + jj * TK + 2 * piece, src[1] + fidx32(N, 1, c - 1, T.j0 + jj, T.k0 + 2 * piece));
            }
            else
            {
                if (first) continue;
                const int w = v - XP - YP, jj = w / FZK, kk = w - jj * FZK;
                cp_async8(dst + FXN + FYN + w, src[2] + fidx32(N, 2, c - 1, T.j0 + jj, T.k0 + kk));
            }
        }
        cp_async_commit();
    };

    double m = 0.0;
    float mf = 0.0f;
    unsigned long long bad = 0;
    load(false, 0, T.i0 - 1);
    load(true, T.i0, T.i0);
    // With the next stage's recovery (NEXT), a plane's face inputs are staged
    // during the previous plane's recovery phase, a whole plane ahead of their
    // use; without it, at the start of their own plane, ahead of the edges.
    if (NEXT) stage_faces(T.i0, true);
    for (int c = T.i0; c <= T.i1; ++c)
    {
        const bool first = c == T.i0, last = c == T.i1;
        cp_async_wait_all();
        __syncthreads();                   // this plane's fields landed; the previous plane's work is done
        if (!NEXT) stage_faces(c, first);
        if (!last) load(true, c + 1, c + 1);
        const int s = c & 1, sp = (c - 1) & 1, ys = mod3(c), yp = mod3(c - 1);
        // edge EMFs at i = c (edge_emf_from_face, scheme_mhd_v1.cpp:76-98; ee_f's order).
        // Thread t forms the E0 edges t (and t + EMF_THREADS), the E1 edge t and
        // the E2 edge t in straight-line code, so that their independent chains
        // interleave.
        {
            const int t = threadIdx.x;
            auto edge0 = [&](int u) {
                const int jj = u / E0K, kk = u - jj * E0K;
                const float* y0 = S.ey[ys][0] + YO - 1;
                const float* z0 = S.ez[ys][0];
                return avg(avg(y0[jj * YK + kk], y0[jj * YK + kk + 1]), avg(z0[jj * ZK + kk], z0[(jj + 1) * ZK + kk]));
            };
            float v0 = 0.0f, w0 = 0.0f, v1 = 0.0f, v2 = 0.0f;
            if (t < E0N) v0 = edge0(t);
            if (t + EMF_THREADS < E0N) w0 = edge0(t + EMF_THREADS);
            if (t < E1N)
            {
                const int jj = t / E1K, kk = t - jj * E1K;
                const float* x1 = S.ex[s][0] + XO - 1;
                const float a = avg(S.ez[yp][1][(jj + 1) * ZK + kk], S.ez[ys][1][(jj + 1) * ZK + kk]);
                const float b = avg(x1[(jj + 1) * XK + kk], x1[(jj + 1) * XK + kk + 1]);
                v1 = avg(a, b);
            }
            if (t < E2N)
            {
                const int jj = t / E2K, kk = t - jj * E2K;
                const float a = avg(S.ex[s][1][jj * XK + XO + kk], S.ex[s][1][(jj + 1) * XK + XO + kk]);
                const float b = avg(S.ey[yp][1][jj * YK + YO + kk], S.ey[ys][1][jj * YK + YO + kk]);
                v2 = avg(a, b);
            }
            if (t < E0N) S.e0[s][t] = v0;
            if (t + EMF_THREADS < E0N) S.e0[s][t + EMF_THREADS] = w0;
            if (t < E1N) S.e1[s][t] = v1;
            if (t < E2N) S.e2[s][t] = v2;
        }
        if (!NEXT)
        {
            if (last) cp_async_wait_all();
            else cp_async_wait_prior();    // the staged faces; the next plane's fields may stay in flight
        }
        __syncthreads();
        // faces: x of layer c (the tile); y and z of plane c-1, with the high
        // neighbour's row and column, which the next-stage cells need. Thread t
        // updates the x face t, the y face t and the z face t, again in
        // straight-line code.
        const double dtdl_d = s_dtdl;
        {
            const int t = threadIdx.x;
            static_assert(FXN <= EMF_THREADS && FYN <= EMF_THREADS && FZN <= EMF_THREADS, "one face of each kind per thread");
            const bool dx = t < FXN;
            const bool dy = !first && t < FYN && (NEXT || t < FXN || T.last_j);
            const int jy = t / TK, ky = t - jy * TK;            // jy = TJ: the high neighbour's face
            const int jz = t / FZK, kz = t - jz * FZK;          // kz = TK: the high neighbour's face
            const bool dz = !first && t < FZN && (NEXT || kz < TK || T.last_k);
            double ox = 0.0, oy = 0.0, oz = 0.0;
            if (dx)
            {
                const double cf = curl_f(S.e2[s][(jy + 1) * E2K + ky], S.e2[s][jy * E2K + ky], S.e1[s][jy * E1K + ky + 1],
                                         S.e1[s][jy * E1K + ky]);
                ox = fma(-cf, dtdl_d, S.bin[t]);
                if (with_avg) ox = half_exact(S.bav[t] + ox);
            }
            if (dy)
            {
                const double cf = curl_f(S.e0[sp][jy * E0K + ky + 1], S.e0[sp][jy * E0K + ky], S.e2[s][jy * E2K + ky],
                                         S.e2[sp][jy * E2K + ky]);
                oy = fma(-cf, dtdl_d, S.bin[FXN + t]);
                if (with_avg) oy = half_exact(S.bav[FXN + t] + oy);
            }
            if (dz)
            {
                const double cf = curl_f(S.e1[s][jz * E1K + kz], S.e1[sp][jz * E1K + kz], S.e0[sp][(jz + 1) * E0K + kz],
                                         S.e0[sp][jz * E0K + kz]);
                oz = fma(-cf, dtdl_d, S.bin[FXN + FYN + t]);
                if (with_avg) oz = half_exact(S.bav[FXN + FYN + t] + oz);
            }
            if (dx)
            {
                S.bx[s][t] = ox;
                if (NEXT) S.bxf[s][t] = d2f(ox);
                if (!last || c == N) A.bf_out[0][fidx32(N, 0, c, T.j0 + jy, T.k0 + ky)] = ox;
            }
            if (dy)
            {
                S.by[t] = oy;
                if (NEXT) S.byf[t] = d2f(oy);
                if (jy < TJ || T.last_j) A.bf_out[1][fidx32(N, 1, c - 1, T.j0 + jy, T.k0 + ky)] = oy;
            }
            if (dz)
            {
                S.bz[t] = oz;
                if (NEXT) S.bzf[t] = d2f(oz);
                if (kz < TK || T.last_k) A.bf_out[2][fidx32(N, 2, c - 1, T.j0 + jz, T.k0 + kz)] = oz;
            }
        }
        if (NEXT)
        {
            __syncthreads();               // every face of plane c has read its staged inputs
            if (!last) stage_faces(c + 1, false);
        }
        if (NEXT && !first)
        {
            // the next stage's primitives of plane c-1 (the primitive kernel's arithmetic)
            float* P = static_cast<float*>(A.P);
            for (int t = threadIdx.x; t < FXN; t += EMF_THREADS)
            {
                const int jj = t / TK, kk = t - jj * TK;
                const int64_t cell = cidx32(N, c - 1, T.j0 + jj, T.k0 + kk);
                Prim<float> p;
                if (recover_mixed<NEXT>(A.next_uc, NN, 1, A.dinc, NN, cell,
                                        cell_field(S.bxf[sp][t], S.bxf[s][t], S.byf[t], S.byf[t + TK],
                                                   S.bzf[jj * FZK + kk], S.bzf[jj * FZK + kk + 1]),
                                        gm, p))
                    ++bad;
                store_cell(P, cell, p);
                mf = fmaxf(mf, fastest_speed(p, gm));
            }
        }
    }
    if (NEXT)
    {
        m = double(mf);
        for (int o = 16; o > 0; o >>= 1)
        {
            m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
            bad += __shfl_xor_sync(0xffffffffu, bad, o);
        }
        if ((threadIdx.x & 31) == 0)
        {
            S.wmax[threadIdx.x >> 5] = m;
            S.wbad[threadIdx.x >> 5] = bad;
        }
        __syncthreads();
        if (threadIdx.x == 0)
        {
            double r = 0.0;
            unsigned long long nbad = 0;
            for (int w = 0; w < EMF_THREADS / 32; ++w)
            {
                r = fmax(r, S.wmax[w]);
                nbad += S.wbad[w];
            }
            atomicMax(&A.clock->amax[A.stage ^ 1], (unsigned long long)__double_as_longlong(r));
            if (nbad) atomicAdd(&A.clock->failures, nbad);
        }
    }
}

__global__ void clock_end_kernel(Clock* clock, int rk_order)
{
    if (threadIdx.x != 0) return;
    const double t = clock->time;
    if (rk_order == 2)
    {
        const double t1 = t + clock->dt[0];
        const double t2 = t1 + clock->dt[1];
        clock->time = t * 0.5 + t2 * (1 - 0.5);
    }
    else
    {
        clock->time = t + clock->dt[0];
    }
    clock->iteration += 1;
}

__global__ void div_b_kernel(int N, const double* b1, const double* b2, const double* b3, unsigned long long* out)
{
    const int64_t NN = int64_t(N) * N * N;
    double m = 0.0;
    for (int64_t c = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; c < NN; c += int64_t(gridDim.x) * blockDim.x)
    {
        int i, j, k;
        unflatten(c, N, N, i, j, k);
        const double d = (b1[fidx(N, 0, i + 1, j, k)] - b1[fidx(N, 0, i, j, k)])
                       + (b2[fidx(N, 1, i, j + 1, k)] - b2[fidx(N, 1, i, j, k)])
                       + (b3[fidx(N, 2, i, j, k + 1)] - b3[fidx(N, 2, i, j, k)]);
        m = fmax(m, fabs(d));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// Initial state (construct_conserved discretisation, src/scheme_mhd_v1.cpp:311-342)
struct Mode { double k[3], phase_v, v[3], phase_a, a[3]; };

__device__ inline void mode_field(const Mode* modes, int count, const double x[3], int which, double amp, double out[3])
{
    out[0] = out[1] = out[2] = 0.0;
    for (int m = 0; m < count; ++m)
    {
        const Mode& t = modes[m];
        const double arg = 2.0 * M_PI * (t.k[0] * x[0] + t.k[1] * x[1] + t.k[2] * x[2]) + (which == 0 ? t.phase_v : t.phase_a);
        const double s = sin(arg);
        for (int c = 0; c < 3; ++c) out[c] += (which == 0 ? t.v[c] : t.a[c]) * s;
    }
    for (int c = 0; c < 3; ++c) out[c] *= amp;
}

__device__ inline double lin(int i, int N) { return 0.0 + (1.0 - 0.0) * double(i) / double(N + 1 - 1); }

__device__ inline double edge_a(const Mode* modes, int count, double a_amp, int N, int axis, int i, int j, int k)
{
    double x[3] = {lin(i, N), lin(j, N), lin(k, N)};
    if (axis == 0) x[0] = 0.5 * (lin(i, N) + lin(i + 1, N));
    if (axis == 1) x[1] = 0.5 * (lin(j, N) + lin(j + 1, N));
    if (axis == 2) x[2] = 0.5 * (lin(k, N) + lin(k + 1, N));
    double A[3];
    mode_field(modes, count, x, 1, a_amp, A);
    return A[axis] * (1.0 / double(N));
}

__global__ void init_faces_kernel(int N, const Mode* modes, int count, double a_amp, double* b1, double* b2, double* b3)
{
    const double dl = 1.0 / double(N);
    const double da = dl * dl;
    const int64_t nf0 = nb(N, 0), nf1 = nb(N, 1), nf2 = nb(N, 2);
    for (int64_t t = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; t < nf0 + nf1 + nf2; t += int64_t(gridDim.x) * blockDim.x)
    {
        int64_t f = t;
        int axis = 0;
        if (f >= nf0) { f -= nf0; axis = 1; if (f >= nf1) { f -= nf1; axis = 2; } }
        int i, j, k;
        const int n1 = N + (axis == 1), n2 = N + (axis == 2);
        unflatten(f, n1, n2, i, j, k);
        auto ae = [&] (int ax, int a, int b, int c) { return edge_a(modes, count, a_amp, N, ax, a, b, c); };
        if (axis == 0)
            b1[f] = ((ae(2, i, j + 1, k) - ae(2, i, j, k)) - (ae(1, i, j, k + 1) - ae(1, i, j, k))) / da;
        else if (axis == 1)
            b2[f] = ((ae(0, i, j, k + 1) - ae(0, i, j, k)) - (ae(2, i + 1, j, k) - ae(2, i, j, k))) / da;
        else
            b3[f] = ((ae(1, i + 1, j, k) - ae(1, i, j, k)) - (ae(0, i, j + 1, k) - ae(0, i, j, k))) / da;
    }
}

__global__ void init_cells_kernel(int N, const Mode* modes, int count, double v_amp, double gm, const double* b1,
                                  const double* b2, const double* b3, double* uc)
{
    const int64_t NN = int64_t(N) * N * N;
    for (int64_t c = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; c < NN; c += int64_t(gridDim.x) * blockDim.x)
    {
        int i, j, k;
        unflatten(c, N, N, i, j, k);
        const double x[3] = {0.5 * (lin(i, N) + lin(i + 1, N)), 0.5 * (lin(j, N) + lin(j + 1, N)), 0.5 * (lin(k, N) + lin(k + 1, N))};
        Prim<double> p;
        p.d = 1.0;
        mode_field(modes, count, x, 0, v_amp, p.v);
        p.p = 1.0;
        p.b[0] = 0.5 * (b1[fidx(N, 0, i, j, k)] + b1[fidx(N, 0, i + 1, j, k)]);
        p.b[1] = 0.5 * (b2[fidx(N, 1, i, j, k)] + b2[fidx(N, 1, i, j + 1, k)]);
        p.b[2] = 0.5 * (b3[fidx(N, 2, i, j, k)] + b3[fidx(N, 2, i, j, k + 1)]);
        double u[5];
        conserved(p, gm, u);
        for (int q = 0; q < 5; ++q) uc[q * NN + c] = u[q];
    }
}

// ---------------------------------------------------------------- host side
struct Workspace
{
    void* P;
    void* F[3];
    void* E[3];
    double* u1;
    double* b1[3];
};

int64_t workspace_bytes(int N, int precision, bool rk2)
{
    const int64_t NN = int64_t(N) * N * N;
    const int64_t NF = nb(N, 0);
    const int64_t r = precision == MARA_MIXED ? 4 : 8;
    // seven 256-byte aligned regions (P, F[3], E[3]) plus alignment slack;
    // each E region holds two components of the larger of the face count and
    // the fused path's padded z rows
    const int64_t NE = std::max(NF, NN + 4 * int64_t(N) * N);
    int64_t bytes = NN * r * 8 + NF * r * 3 * 5 + NE * r * 3 * 2 + 8 * 256;
    if (rk2) bytes += 8 * (5 * NN + nb(N, 0) + nb(N, 1) + nb(N, 2));
    return bytes + 256;
}

Workspace carve(void* base, int N, int precision, bool rk2)
{
    const int64_t NN = int64_t(N) * N * N;
    const int64_t r = precision == MARA_MIXED ? 4 : 8;
    char* p = static_cast<char*>(base);
    const int64_t NF = nb(N, 0);   // every face array has (N+1) N^2 entries
    auto up = [] (char* q) { return reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(q) + 255) & ~uintptr_t(255)); };
    Workspace w{};
    w.P = up(p); p = up(static_cast<char*>(w.P) + 8 * NN * r);     // 16-byte vector records need alignment
    for (int a = 0; a < 3; ++a) { w.F[a] = p; p = up(p + 5 * NF * r); }
    const int64_t NE = std::max(NF, NN + 4 * int64_t(N) * N);   // see workspace_bytes
    for (int a = 0; a < 3; ++a) { w.E[a] = p; p = up(p + 2 * NE * r); }
    if (rk2)
    {
        w.u1 = reinterpret_cast<double*>(p); p += 5 * NN * 8;
        for (int a = 0; a < 3; ++a) { w.b1[a] = reinterpret_cast<double*>(p); p += nb(N, a) * 8; }
    }
    return w;
}

int check(const mara_mhd_params* mp)
{
    MARA_REQUIRE(mp != nullptr, "mhd: params is null");
    MARA_REQUIRE(mp->N >= 4 && mp->N <= 1024, "mhd: N must be in [4, 1024]");
    MARA_REQUIRE(mp->gamma_law_index > 1.0, "mhd: gamma_law_index must exceed 1");
    MARA_REQUIRE(mp->cfl > 0.0, "mhd: cfl must be positive");
    return MARA_OK;
}

inline int blocks_for(int64_t n) { return int(std::min<int64_t>((n + 255) / 256, 152 * 16)); }

// The fused mixed stage (flux_kernel + emf_kernel): 1 = on wherever the
// mesh allows it (N a multiple of 32), 0 = the face and update kernels.
// g_ct_chunks > 0 fixes the number of i chunks; 0 chooses it from the SM count.
std::atomic<int> g_ct_fused{1};
std::atomic<int> g_ct_chunks{0};

inline bool fused_path(int precision, int N)
{
    return precision == MARA_MIXED && g_ct_fused.load(std::memory_order_relaxed) && N % fused::TK == 0;
}

Args stage_args(const mara_mhd_params* mp, const Workspace& w, Clock* clock, int st, const double* u_in, int64_t ucs,
                int64_t uzs, const double* const b_in[3], const double* uavg, const double* const bavg[3],
                double* u_out, double* const b_out[3])
{
    const int N = mp->N;
    Args A;
    std::memset(&A, 0, sizeof A);
    A.N = N;
    A.div_n = fast_div(uint32_t(N));
    A.div_n1 = fast_div(uint32_t(N + 1));
    A.div_nn = fast_div(uint32_t(N) * uint32_t(N));
    A.div_nn1 = fast_div(uint32_t(N) * uint32_t(N + 1));
    A.gamma = mp->gamma_law_index;
    A.dl = 1.0 / double(N);
    A.cfl = mp->cfl;
    A.theta = mp->plm_theta;
    A.uc = u_in;
    A.ucs = ucs;
    A.uzs = uzs;
    A.uavg = uavg;
    A.uc_out = u_out;
    for (int a = 0; a < 3; ++a)
    {
        A.bf[a] = b_in[a];
        A.bavg[a] = bavg ? bavg[a] : nullptr;
        A.bf_out[a] = b_out[a];
        A.F[a] = w.F[a];
        A.E[a] = w.E[a];
    }
    A.P = w.P;
    A.clock = clock;
    A.stage = st;
    A.dinc = reinterpret_cast<float*>(w.u1);   // the FP32 increments reuse the stage-1 state region
    return A;
}

template<typename R>
int launch_prim(const Args& A, int mixed_mode, cudaStream_t s)
{
    const int64_t NN = int64_t(A.N) * A.N * A.N;
    if constexpr (sizeof(R) == sizeof(float))
    {
        if (mixed_mode == MIX_INCREMENT) prim_kernel<R, MIX_INCREMENT><<<blocks_for(NN), 256, 0, s>>>(A);
        else if (mixed_mode == MIX_FROM_INCREMENT) prim_kernel<R, MIX_FROM_INCREMENT><<<blocks_for(NN), 256, 0, s>>>(A);
        else prim_kernel<R, MIX_PLAIN><<<blocks_for(NN), 256, 0, s>>>(A);
    }
    else prim_kernel<R, MIX_PLAIN><<<blocks_for(NN), 256, 0, s>>>(A);
    return launch_status("mhd prim_kernel");
}

// One stage: u_out/b_out = advance_mhd_ct(u_in/b_in) [averaged with avg].
template<typename R>
int stage(const mara_mhd_params* mp, const Workspace& w, Clock* clock, int st,
          const double* u_in, int64_t ucs, int64_t uzs, const double* const b_in[3],
          const double* uavg, const double* const bavg[3], double* u_out, double* const b_out[3],
          int mixed_mode, cudaStream_t s)
{
    const int N = mp->N;
    const int64_t NN = int64_t(N) * N * N;
    const Args A = stage_args(mp, w, clock, st, u_in, ucs, uzs, b_in, uavg, bavg, u_out, b_out);
    if (int r = launch_prim<R>(A, mixed_mode, s)) return r;
    dt_kernel<<<1, 32, 0, s>>>(clock, st, mp->cfl, A.dl, 0);
    if (int r = launch_status("mhd dt_kernel")) return r;
    face_kernel<R, 0><<<blocks_for(nb(N, 0)), 256, 0, s>>>(A);
    face_kernel<R, 1><<<blocks_for(nb(N, 1)), 256, 0, s>>>(A);
    face_kernel<R, 2><<<blocks_for(nb(N, 2)), 256, 0, s>>>(A);
    if (int r = launch_status("mhd face_kernel")) return r;
    const int ub = blocks_for(NN), fb = blocks_for(nb(N, 0) + nb(N, 1) + nb(N, 2));
    if constexpr (sizeof(R) == sizeof(float))
    {
        if (mixed_mode == MIX_INCREMENT) update_kernel<R, MIX_INCREMENT, 0><<<ub, 256, 0, s>>>(A);
        else if (mixed_mode == MIX_FROM_INCREMENT) update_kernel<R, MIX_FROM_INCREMENT, 0><<<ub, 256, 0, s>>>(A);
        else update_kernel<R, MIX_PLAIN, 0><<<ub, 256, 0, s>>>(A);
    }
    else update_kernel<R, MIX_PLAIN, 0><<<ub, 256, 0, s>>>(A);
    if (int r = launch_status("mhd update_kernel (cells)")) return r;
    update_kernel<R, MIX_PLAIN, 1><<<fb, 256, 0, s>>>(A);
    return launch_status("mhd update_kernel (faces)");
}

// Dynamic shared memory of the EMF kernel (above the 48 KB of a static
// allocation), allowed once per device and instantiation
template<int NEXT>
int emf_attribute(int dev)
{
    static PerDeviceOnce once;
    return once.run(dev, []() -> int {
        MARA_CUDA(cudaFuncSetAttribute(emf_kernel<NEXT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       int(sizeof(fused::EmfSmem))));
        return MARA_OK;
    });
}

// i chunks of a fused kernel: at least two waves of resident blocks and at
// most 16 planes per chunk (blocks of equal work finish in waves, and a short
// last wave of long blocks leaves most SMs idle; measured at 128^3 and 256^3),
// at least four planes per chunk (each chunk solves one extra layer of faces)
// (WHICH keeps one occupancy cache per kernel: both kernels have the same
// function type, so the type alone would share one)
template<int WHICH, typename K>
int fused_chunks(K kernel, int threads, size_t smem, int N, int* chunks)
{
    static PerDeviceOnce once;
    static int slots[64] = {};
    int dev = 0;
    MARA_CUDA(cudaGetDevice(&dev));
    if (int r = once.run(dev, [&]() -> int {
            int b = 0, n = 0;
            MARA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, threads, smem));
            MARA_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
            slots[dev & 63] = n * (b > 0 ? b : 1);
            return MARA_OK;
        }))
        return r;
    const int tiles = (N / fused::TJ) * (N / fused::TK);
    int c = g_ct_chunks.load(std::memory_order_relaxed);
    if (c <= 0) c = std::max(1, std::min(N / 4, std::max(N / 16, (2 * slots[dev & 63] + tiles - 1) / tiles)));
    *chunks = std::min(c, N);
    return MARA_OK;
}

// The fused mixed stage: [primitives,] dt, flux_kernel, emf_kernel. `next`
// (0, MIX_INCREMENT or MIX_FROM_INCREMENT) makes the EMF kernel recover the
// next stage's primitives from next_uc (and its maximum wavespeed), so that
// the next stage runs with need_prim = false. b_out must not alias b_in or
// bavg: the EMF kernel re-solves the faces its tile's cells share with the
// neighbouring tiles and reads their inputs while the owners write.
int stage_fused(const mara_mhd_params* mp, const Workspace& w, Clock* clock, int st, const double* u_in, int64_t ucs,
                int64_t uzs, const double* const b_in[3], const double* const bavg[3], double* u_out,
                double* const b_out[3], int mixed_mode, bool need_prim, int next, const double* next_uc,
                cudaStream_t s)
{
    const int N = mp->N;
    Args A = stage_args(mp, w, clock, st, u_in, ucs, uzs, b_in, nullptr, bavg, u_out, b_out);
    A.next_uc = next_uc;
    if (need_prim)
        if (int r = launch_prim<float>(A, mixed_mode, s)) return r;
    dt_kernel<<<1, 32, 0, s>>>(clock, st, mp->cfl, A.dl, 0);
    if (int r = launch_status("mhd dt_kernel")) return r;
    const int tiles = (N / fused::TJ) * (N / fused::TK);
    int cf = 0, ce = 0, dev = 0;
    const size_t esm = sizeof(fused::EmfSmem);
    MARA_CUDA(cudaGetDevice(&dev));
    if (int r = emf_attribute<0>(dev)) return r;
    if (int r = emf_attribute<MIX_INCREMENT>(dev)) return r;
    if (int r = emf_attribute<MIX_FROM_INCREMENT>(dev)) return r;
    if (int r = fused_chunks<0>(flux_kernel<MIX_FROM_INCREMENT>, fused::FLUX_THREADS, 0, N, &cf)) return r;
    if (int r = fused_chunks<1>(emf_kernel<MIX_INCREMENT>, fused::EMF_THREADS, esm, N, &ce)) return r;
    if (mixed_mode == MIX_INCREMENT) flux_kernel<MIX_INCREMENT><<<tiles * cf, fused::FLUX_THREADS, 0, s>>>(A, cf);
    else if (mixed_mode == MIX_FROM_INCREMENT) flux_kernel<MIX_FROM_INCREMENT><<<tiles * cf, fused::FLUX_THREADS, 0, s>>>(A, cf);
    else flux_kernel<MIX_PLAIN><<<tiles * cf, fused::FLUX_THREADS, 0, s>>>(A, cf);
    if (int r = launch_status("mhd flux_kernel")) return r;
    if (next == MIX_INCREMENT) emf_kernel<MIX_INCREMENT><<<tiles * ce, fused::EMF_THREADS, esm, s>>>(A, ce);
    else if (next == MIX_FROM_INCREMENT) emf_kernel<MIX_FROM_INCREMENT><<<tiles * ce, fused::EMF_THREADS, esm, s>>>(A, ce);
    else emf_kernel<0><<<tiles * ce, fused::EMF_THREADS, esm, s>>>(A, ce);
    return launch_status("mhd emf_kernel");
}

int run_stage(int precision, const mara_mhd_params* mp, const Workspace& w, Clock* clock, int st,
              const double* u_in, int64_t ucs, int64_t uzs, const double* const b_in[3], const double* uavg,
              const double* const bavg[3], double* u_out, double* const b_out[3], cudaStream_t s)
{
    if (precision == MARA_MIXED)
        return stage<float>(mp, w, clock, st, u_in, ucs, uzs, b_in, uavg, bavg, u_out, b_out, MIX_PLAIN, s);
    return stage<double>(mp, w, clock, st, u_in, ucs, uzs, b_in, uavg, bavg, u_out, b_out, MIX_PLAIN, s);
}

} // namespace mhd
} // namespace mara

using namespace mara;
using namespace mara::mhd;

extern "C" {

int64_t mara_mhd_clock_bytes(void) { return int64_t(sizeof(Clock)); }

int mara_mhd_fused_stage(int32_t enable, int32_t chunks)
{
    MARA_REQUIRE(enable == 0 || enable == 1, "mara_mhd_fused_stage: enable must be 0 or 1");
    MARA_REQUIRE(chunks >= 0 && chunks <= 1024, "mara_mhd_fused_stage: chunks must be in [0, 1024]");
    g_ct_fused.store(enable);
    g_ct_chunks.store(chunks);
    return MARA_OK;
}

int64_t mara_mhd_workspace_bytes(const mara_mhd_params* mp, int32_t rk_order, int32_t precision)
{
    if (check(mp)) return -1;
    return workspace_bytes(mp->N, precision, rk_order == 2);
}

int mara_mhd_clock_init(void* clock, double time, void* stream)
{
    MARA_REQUIRE(clock != nullptr, "mara_mhd_clock_init: clock is null");
    Clock c;
    std::memset(&c, 0, sizeof c);
    c.time = time;
    cudaStream_t s = as_stream(stream);
    MARA_CUDA(cudaMemcpyAsync(clock, &c, sizeof c, cudaMemcpyHostToDevice, s));
    MARA_CUDA(cudaStreamSynchronize(s));
    return MARA_OK;
}

int mara_mhd_advance_ct(const mara_mhd_params* mp, const double* uc, int64_t component_stride, int64_t cell_stride,
                        const double* bf1, const double* bf2, const double* bf3, double* uc_out, double* bf1_out,
                        double* bf2_out, double* bf3_out, void* clock, int32_t precision, void* workspace,
                        void* stream)
{
    if (int r = check(mp)) return r;
    MARA_REQUIRE(uc && bf1 && bf2 && bf3 && uc_out && bf1_out && bf2_out && bf3_out && clock && workspace,
                 "mara_mhd_advance_ct: null buffer");
    MARA_REQUIRE(precision == MARA_FP64 || precision == MARA_MIXED, "mara_mhd_advance_ct: bad precision");
    MARA_REQUIRE(uc_out != uc && bf1_out != bf1 && bf2_out != bf2 && bf3_out != bf3,
                 "mara_mhd_advance_ct: outputs must not alias inputs");
    cudaStream_t s = as_stream(stream);
    Clock* c = static_cast<Clock*>(clock);
    Workspace w = carve(workspace, mp->N, precision, false);
    const double* b_in[3] = {bf1, bf2, bf3};
    double* b_out[3] = {bf1_out, bf2_out, bf3_out};
    dt_kernel<<<1, 32, 0, s>>>(c, 0, mp->cfl, 1.0 / mp->N, 1);
    if (int r = launch_status("mhd dt_kernel")) return r;
    if (fused_path(precision, mp->N))
    {
        if (int r = stage_fused(mp, w, c, 0, uc, component_stride, cell_stride, b_in, nullptr, uc_out, b_out, MIX_PLAIN,
                                true, 0, nullptr, s))
            return r;
    }
    else if (int r = run_stage(precision, mp, w, c, 0, uc, component_stride, cell_stride, b_in, nullptr, nullptr, uc_out,
                               b_out, s))
        return r;
    clock_end_kernel<<<1, 32, 0, s>>>(c, 1);
    return launch_status("mhd clock_end_kernel");
}

int mara_mhd_advance(const mara_mhd_params* mp, double* uc, double* bf1, double* bf2, double* bf3, void* clock,
                     int32_t steps, int32_t rk_order, int32_t precision, void* workspace, void* stream)
{
    if (int r = check(mp)) return r;
    MARA_REQUIRE(uc && bf1 && bf2 && bf3 && clock && workspace, "mara_mhd_advance: null buffer");
    MARA_REQUIRE(rk_order == 1 || rk_order == 2, "mara_mhd_advance: rk_order must be 1 or 2");
    MARA_REQUIRE(precision == MARA_FP64 || precision == MARA_MIXED, "mara_mhd_advance: bad precision");
    MARA_REQUIRE(steps >= 0, "mara_mhd_advance: negative step count");
    MARA_REQUIRE(rk_order == 2, "mara_mhd_advance: in-place forward Euler is not supported; use mara_mhd_advance_ct");
    cudaStream_t s = as_stream(stream);
    Clock* c = static_cast<Clock*>(clock);
    Workspace w = carve(workspace, mp->N, precision, true);
    const int64_t NN = int64_t(mp->N) * mp->N * mp->N;
    double* b0[3] = {bf1, bf2, bf3};
    const double* b0c[3] = {bf1, bf2, bf3};
    const double* b1c[3] = {w.b1[0], w.b1[1], w.b1[2]};
    if (steps > 0 && fused_path(precision, mp->N))
    {
        // Fused mixed RK2. Stage 2 may not write B over its averaging partner
        // (stage_fused), so the face fields alternate between the caller's
        // arrays and scratch in the (here unused) flux arrays of the
        // workspace, and come back to the caller's arrays at the end.
        double* X[3] = {static_cast<double*>(w.F[0]), static_cast<double*>(w.F[1]), static_cast<double*>(w.F[2])};
        bool in_caller = true;
        dt_kernel<<<1, 32, 0, s>>>(c, 0, mp->cfl, 1.0 / mp->N, 1);
        if (int r = launch_status("mhd dt_kernel")) return r;
        for (int step = 0; step < steps; ++step)
        {
            double* const* cur = in_caller ? b0 : X;
            double* const* nxt = in_caller ? X : b0;
            const double* curc[3] = {cur[0], cur[1], cur[2]};
            if (int r = stage_fused(mp, w, c, 0, uc, NN, 1, curc, nullptr, nullptr, w.b1, MIX_INCREMENT, step == 0,
                                    MIX_FROM_INCREMENT, uc, s))
                return r;
            if (int r = stage_fused(mp, w, c, 1, uc, NN, 1, b1c, curc, uc, nxt, MIX_FROM_INCREMENT, false,
                                    step + 1 < steps ? MIX_INCREMENT : 0, uc, s))
                return r;
            clock_end_kernel<<<1, 32, 0, s>>>(c, 2);
            if (int r = launch_status("mhd clock_end_kernel")) return r;
            in_caller = !in_caller;
        }
        if (!in_caller)
            for (int a = 0; a < 3; ++a)
                MARA_CUDA(cudaMemcpyAsync(b0[a], X[a], sizeof(double) * size_t(nb(mp->N, a)), cudaMemcpyDeviceToDevice, s));
        return MARA_OK;
    }
    for (int step = 0; step < steps; ++step)
    {
        dt_kernel<<<1, 32, 0, s>>>(c, 0, mp->cfl, 1.0 / mp->N, 1);
        if (int r = launch_status("mhd dt_kernel")) return r;
        if (precision == MARA_MIXED)
        {
            // stage 1: b1 = advance(b0) in FP64; the cells keep only the FP32
            // increment d1 = u1 - u0. Stage 2 reads u1 as u0 + d1 and writes
            // u0 + (d1 + d2) / 2, which is u0/2 + (u1 + d2)/2 to FP32 rounding
            // of the increments.
            if (int r = stage<float>(mp, w, c, 0, uc, NN, 1, b0c, nullptr, nullptr, nullptr, w.b1, MIX_INCREMENT, s))
                return r;
            if (int r = stage<float>(mp, w, c, 1, uc, NN, 1, b1c, nullptr, b0c, uc, b0, MIX_FROM_INCREMENT, s))
                return r;
        }
        else
        {
            // stage 1: (u1, b1) = advance_mhd_ct(u0, b0) with its own dt
            if (int r = run_stage(precision, mp, w, c, 0, uc, NN, 1, b0c, nullptr, nullptr, w.u1, w.b1, s)) return r;
            // stage 2: u0 <- u0/2 + advance_mhd_ct(u1, b1)/2, in place (each element reads its own u0)
            if (int r = run_stage(precision, mp, w, c, 1, w.u1, NN, 1, b1c, uc, b0c, uc, b0, s)) return r;
        }
        clock_end_kernel<<<1, 32, 0, s>>>(c, 2);
        if (int r = launch_status("mhd clock_end_kernel")) return r;
    }
    return MARA_OK;
}

int mara_mhd_mode_table(uint64_t seed, int32_t modes, double* table)
{
    MARA_REQUIRE(modes > 0 && modes <= 4096 && table, "mara_mhd_mode_table: bad argument");
    auto hash = [seed] (uint64_t i) {
        uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return z;
    };
    auto uni = [&] (uint64_t i) { return double(hash(i) >> 11) * 0x1.0p-53; };
    uint64_t counter = 0;
    for (int m = 0; m < modes; ++m)
    {
        double k[3];
        for (int attempt = 0;; ++attempt)
        {
            for (int c = 0; c < 3; ++c) k[c] = double(int(hash(counter++) % 9) - 4);
            const double kk = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
            if (kk > 0.0 && kk <= 16.0) break;
            if (attempt > 10000) return fail(MARA_ERR_NUMERIC, "mara_mhd_mode_table: no admissible wavevector");
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
        // polarisation of A transverse to k, scaled by 1/|k| so every mode of B = curl A has unit amplitude / 2pi
        double r[3];
        double a[3], norm2 = 0.0;
        do {
            unit(r);
            const double rk = (r[0] * k[0] + r[1] * k[1] + r[2] * k[2]) / (kn * kn);
            norm2 = 0.0;
            for (int c = 0; c < 3; ++c) { a[c] = r[c] - rk * k[c]; norm2 += a[c] * a[c]; }
        } while (norm2 < 1e-6);
        for (int c = 0; c < 3; ++c) t[8 + c] = a[c] / (std::sqrt(norm2) * kn);
    }
    return MARA_OK;
}

int mara_mhd_initial_state(const mara_mhd_params* mp, const double* table, int32_t modes, double v_amp, double a_amp,
                           double* uc, double* bf1, double* bf2, double* bf3, void* workspace, void* stream)
{
    if (int r = check(mp)) return r;
    MARA_REQUIRE(table && modes > 0 && uc && bf1 && bf2 && bf3 && workspace, "mara_mhd_initial_state: bad argument");
    cudaStream_t s = as_stream(stream);
    // the mode table goes through the caller's workspace (no allocation)
    MARA_CUDA(cudaMemcpyAsync(workspace, table, sizeof(double) * 11 * modes, cudaMemcpyHostToDevice, s));
    MARA_CUDA(cudaStreamSynchronize(s));
    const Mode* m = static_cast<const Mode*>(workspace);
    const int N = mp->N;
    init_faces_kernel<<<blocks_for(nb(N, 0) * 3), 256, 0, s>>>(N, m, modes, a_amp, bf1, bf2, bf3);
    if (int r = launch_status("mhd init_faces_kernel")) return r;
    init_cells_kernel<<<blocks_for(int64_t(N) * N * N), 256, 0, s>>>(N, m, modes, v_amp, mp->gamma_law_index, bf1, bf2,
                                                                     bf3, uc);
    return launch_status("mhd init_cells_kernel");
}

int mara_mhd_max_div_b(const mara_mhd_params* mp, const double* bf1, const double* bf2, const double* bf3,
                       double* out, void* stream)
{
    if (int r = check(mp)) return r;
    MARA_REQUIRE(bf1 && bf2 && bf3 && out, "mara_mhd_max_div_b: null buffer");
    cudaStream_t s = as_stream(stream);
    MARA_CUDA(cudaMemsetAsync(out, 0, sizeof(double), s));
    div_b_kernel<<<blocks_for(int64_t(mp->N) * mp->N * mp->N), 256, 0, s>>>(
        mp->N, bf1, bf2, bf3, reinterpret_cast<unsigned long long*>(out));
    return launch_status("mhd div_b_kernel");
}

} // extern "C"
