// Device-side pieces of the minidisk Godunov update shared by the
// single-mesh kernels (minidisk.cu) and the batched ensemble (ensemble.cu):
// the launch arguments, the mixed-precision conversions and fast math, PLM
// slopes, the HLLE + viscous face flux, the mixed cell update and the
// warp-strip sweep of one strip segment.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>
#include "common.cuh"
#include "mixed_math.cuh"

namespace mara {
namespace md {

constexpr int TX = 16, TY = 32, NT = 256;
constexpr int EX = TX + 4, EY = TY + 4;     // halo tile
constexpr int GX = TX + 2, GY = TY + 2;     // slope region
constexpr int NFX = (TX + 1) * TY;          // x faces
constexpr int NFY = TX * (TY + 1);          // y faces

// Stage kinds: plain FP64; mixed stage writing an FP64 state from its input
// (forward Euler, or the tiled kernel's stage 1 of RK2 when d_out is set);
// mixed stage 2 of RK2; the per-block drop-in; mixed stage 1 of RK2 writing
// only the FP32 increment (the sweeps' form of it, with no state operands).
enum Kind { K_FP64 = 0, K_MIX1 = 1, K_MIX2 = 2, K_BLOCK = 3, K_MIXD = 4 };

// Single-precision constants of the mixed path, prepared on the host so that
// no FP64 instruction (GB300 runs FP64 at 1/64 of the FP32 rate) is issued
// for them on the device.
struct FloatConsts
{
    float rs2, inv_mach2, half_nu, half_inv_dl, quarter_inv_dl, inv_dl, theta, two_theta, R, dl;
    float sink_rate, inv_s6, buffer_rate, neg2_inv_buffer_scale, omega, omega2, two_omega;
    float inv_mach;         // 1 / M: the sound speed is sqrt(pot) / M, pot = 1/sqrt(r^2 + rs^2)
    float visc_mu;          // nu / 2 / (4 dl): the viscous coefficient per (Sigma_l + Sigma_r) of doubled slopes
    float sink_ex2;         // -log2(e) / s^6: sink rate = sink_rate 2^(q^3 sink_ex2), q = |x - x_body|^2
    float buffer_ex2;       // -2 log2(e) / buffer_scale
    float sink_far;         // q at and beyond which 2^(q^3 sink_ex2) is below the smallest normal float: exactly 0
};

struct Args
{
    int N;                 // cells per side of the mesh (K_BLOCK: block size)
    int n;                 // block size (zones per block side)
    int level;             // block level (2^level blocks per side)
    int tiles_y;
    int sweep_rows;        // mixed sweep: rows per warp
    int use_tma;           // FP64 tiles: interior halo tiles by one TMA copy
    uint64_t bi, bj;       // K_BLOCK: block coordinates
    double R, dl;
    double rs2;            // softening_length^2 (std::pow(rs, 2.0) on the host)
    double mach, nu, omega, sink_rate, s6, buffer_rate, buffer_scale, theta;
    double dt;             // used when clock == nullptr
    double bin[6];         // m1, x1, y1, m2, x2, y2; used when clock == nullptr
    const mara_minidisk_clock* clock;
    int stage;             // which clock->binary row this stage uses
    const double* u_in;    // FP64/MIX: stage state (FP64) or u0; K_BLOCK: uc AoS
    const double* u_avg;   // K_FP64: optional RK2 average partner
    const float* d1;       // K_MIX2: FP32 stage-1 increment
    double* u_out;         // FP64 result
    float* d_out;          // K_MIX1 + RK2: increment out
    const double* pe;      // K_BLOCK: (n+4)^2 AoS primitives
    unsigned long long* amax;  // optional: max fastest wavespeed of u_out (double bits)
    int amax_key;          // mixed kinds: 1 = write the speed key of the fastest cell (speed_key) instead
    double* diag;          // optional: rate row of this stage (diagnostic sums 0..12 of the stage input)
    FloatConsts f;
    // Mixed RK2 sweeps: block 0 of the launch takes the binaries off the
    // critical path (side_binary_job). 1 (stage 1): two warps solve, side by
    // side, the stage-2 binary at t + dt into clock->binary[1] and the next
    // step's stage-1 binary at the RK2 end time into next_binary (stage 1
    // itself reads binary[0]); 2 (stage 2, which reads binary[1]): copy
    // next_binary into clock->binary[0]. 0 = none.
    int side_binary;
    double* next_binary;   // 6 doubles of workspace for side_binary
    double mass_ratio, eccentricity;
};

// Diagnostic sums taken per cell (the rate-vector entries 0..12 of
// mara_minidisk_diagnostics); 13..15 follow from them in the clock kernel.
constexpr int DIAG_SUMS = 13;

// ------------------------------------------------------------- geometry
// vertex_positions (problems/minidisk_scheme.cpp:101-116): linspace of block b
__host__ __device__ inline double vertex(double R, int n, int level, uint64_t b, int k)
{
    double dlv = double(1 << level);
    double x0 = R * (-1 + double(2 * b) / dlv);
    double x1 = R * (-1 + double(2 * (b + 1)) / dlv);
    return x0 + (x1 - x0) * double(k) / double(n);
}

__device__ inline int wrap(int g, int N)
{
    g %= N;
    return g < 0 ? g + N : g;
}

// ------------------------------------------------------------- PLM
// Generalised minmod on unit spacing (scheme_plm_gradient.hpp:56-63). The
// reference's 0.25*|sa+sb|*(sa+sc)*min(|a|,|b|,|c|) equals copysign(min, a)
// when a, b, c share a sign and zero otherwise; that is what is computed here.
__device__ inline double plm(double yl, double y0, double yr, double theta)
{
    double a = (y0 - yl) * theta;
    double b = (yr - yl) * 0.5;
    double c = (yr - y0) * theta;
    double m = fmin(fmin(fabs(a), fabs(b)), fabs(c));
    long long sa = __double_as_longlong(a), sb = __double_as_longlong(b), sc = __double_as_longlong(c);
    return ((sa ^ sb) | (sa ^ sc)) < 0 ? 0.0 : copysign(m, a);
}

// ------------------------------------------------------------- FP32 lanes
// The mixed path is written once for T = float (one column per thread) and
// T = float2 (two adjacent columns per thread). Every operation is explicit
// and rounded to nearest, with no contraction left to the compiler, so both
// forms (and every kernel built from them) give bit-identical results. The
// pair form issues two scalar instructions per operation: packed FP32x2
// instructions were measured at most 3% faster here, and did not reproduce
// the scalar rounding inside these kernels.
__device__ __forceinline__ float vadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float vsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float vmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float vfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float vneg(float a) { return -a; }
__device__ __forceinline__ float2 vadd(float2 a, float2 b) { return make_float2(vadd(a.x, b.x), vadd(a.y, b.y)); }
__device__ __forceinline__ float2 vsub(float2 a, float2 b) { return make_float2(vsub(a.x, b.x), vsub(a.y, b.y)); }
__device__ __forceinline__ float2 vmul(float2 a, float2 b) { return make_float2(vmul(a.x, b.x), vmul(a.y, b.y)); }
__device__ __forceinline__ float2 vfma(float2 a, float2 b, float2 c)
{
    return make_float2(vfma(a.x, b.x, c.x), vfma(a.y, b.y, c.y));
}
__device__ __forceinline__ float2 vneg(float2 a) { return make_float2(-a.x, -a.y); }

template<typename T> __device__ __forceinline__ T bc(float c);
template<> __device__ __forceinline__ float bc<float>(float c) { return c; }
template<> __device__ __forceinline__ float2 bc<float2>(float c) { return make_float2(c, c); }

#define MARA_LANEWISE(name, expr)                                                                     \
    __device__ __forceinline__ float name(float a) { return expr(a); }                               \
    __device__ __forceinline__ float2 name(float2 a) { return make_float2(expr(a.x), expr(a.y)); }
MARA_LANEWISE(vrcp, rcp_fast)
MARA_LANEWISE(vsqrt, sqrt_fast)
MARA_LANEWISE(vrsqrt, rsqrt_fast)
#undef MARA_LANEWISE

__device__ __forceinline__ float ex2_fast(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
template<typename T>
__device__ __forceinline__ T vex2(T a)
{
    if constexpr (sizeof(T) == sizeof(float)) return ex2_fast(a);
    else return make_float2(ex2_fast(a.x), ex2_fast(a.y));
}
template<typename T>
__device__ __forceinline__ T vexp(T a)
{
    const T t = vmul(a, bc<T>(1.4426950408889634f));
    if constexpr (sizeof(T) == sizeof(float)) return ex2_fast(t);
    else return make_float2(ex2_fast(t.x), ex2_fast(t.y));
}
__device__ __forceinline__ float vmax(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ float vmin(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ float2 vmax(float2 a, float2 b) { return make_float2(fmaxf(a.x, b.x), fmaxf(a.y, b.y)); }
__device__ __forceinline__ float2 vmin(float2 a, float2 b) { return make_float2(fminf(a.x, b.x), fminf(a.y, b.y)); }

// The FP32 slopes are kept DOUBLED: for a = y0 - yl, b = yr - yl, c = yr - y0,
// 2 minmod(theta a, b / 2, theta c) = minmod(x, b, z) with x = 2 theta a,
// z = 2 theta c (plm_gradient_scalar_t, scheme_plm_gradient.hpp:44-67);
// consumers take a quarter of it for the face values. The three-argument
// minmod is a median, max(min(x, b, z), min(max(x, b, z), 0)): the smallest
// when all three are positive, the largest when all are negative, else zero.
// Scaling by 2 theta and taking minima commute with rounding, so this is
// exactly twice the three-multiply slope (only the sign of a zero result can
// differ from a sign-bit test).
__device__ __forceinline__ float minmod2(float a, float b, float c, float two_theta)
{
    const float x = vmul(two_theta, a), z = vmul(two_theta, c);
    return fmaxf(min3f(x, b, z), fminf(max3f(x, b, z), 0.0f));
}

template<typename T>
__device__ __forceinline__ T vplm2(T yl, T y0, T yr, float two_theta)
{
    const T a = vsub(y0, yl), b = vsub(yr, yl), c = vsub(yr, y0);
    if constexpr (sizeof(T) == sizeof(float)) return minmod2(a, b, c, two_theta);
    else return make_float2(minmod2(a.x, b.x, c.x, two_theta), minmod2(a.y, b.y, c.y, two_theta));
}

// The limited slope of a component: FP64 as the reference has it; FP32
// doubled (vplm2).
template<typename R> __device__ inline R cell_slope(R yl, R y0, R yr, const Args& A);
template<> __device__ inline double cell_slope<double>(double yl, double y0, double yr, const Args& A)
{
    return plm(yl, y0, yr, A.theta);
}
template<> __device__ inline float cell_slope<float>(float yl, float y0, float yr, const Args& A)
{
    return vplm2(yl, y0, yr, A.f.two_theta);
}

// ------------------------------------------------------------- face flux
// HLLE flux (physics_iso2d.hpp:156-173) plus viscous stress
// (problems/minidisk_scheme.cpp:242-281) at one face. pa/pb: left/right cell
// primitives; ga/gb: their slopes along the face normal; ta/tb: transverse.
template<int AXIS>
__device__ inline void face_flux(const double pa[3], const double pb[3], const double ga[3], const double gb[3],
                                 const double ta[3], const double tb[3], double x, double y,
                                 const Args& A, double F[3])
{
    double L[3], Rr[3];
    for (int k = 0; k < 3; ++k)
    {
        L[k] = pa[k] + 0.5 * ga[k];     // (pc + g/2) of the left cell
        Rr[k] = pb[k] - 0.5 * gb[k];    // (pc - g/2) of the right cell
    }
    // sound_speed_squared at the face (problems/minidisk_scheme.cpp:127-132)
    double ph = -1.0 / sqrt((x * x + y * y) + A.rs2);
    double cs2 = -ph / A.mach / A.mach;
    double cs = sqrt(cs2);
    double vl = AXIS == 0 ? L[1] : L[2];
    double vr = AXIS == 0 ? Rr[1] : Rr[2];
    double ul[3] = {L[0], L[0] * L[1], L[0] * L[2]};
    double ur[3] = {Rr[0], Rr[0] * Rr[1], Rr[0] * Rr[2]};
    double pgl = L[0] * cs2, pgr = Rr[0] * cs2;
    double fl[3] = {vl * ul[0], vl * ul[1] + (AXIS == 0 ? pgl : 0.0), vl * ul[2] + (AXIS == 0 ? 0.0 : pgl)};
    double fr[3] = {vr * ur[0], vr * ur[1] + (AXIS == 0 ? pgr : 0.0), vr * ur[2] + (AXIS == 0 ? 0.0 : pgr)};
    double ap = fmax(0.0, fmax(vl + cs, vr + cs));
    double am = fmin(0.0, fmin(vl - cs, vr - cs));
    for (int k = 0; k < 3; ++k)
        F[k] = (ap * fl[k] - am * fr[k] - (ul[k] - ur[k]) * ap * am) / (ap - am);

    if (A.nu != 0.0)
    {
        double mu = A.nu * 0.5 * (Rr[0] + L[0]);
        double vx_long = 0.5 * (ga[1] + gb[1]) / A.dl;
        double vy_long = 0.5 * (ga[2] + gb[2]) / A.dl;
        double vx_tran = 0.5 * (ta[1] + tb[1]) / A.dl;
        double vy_tran = 0.5 * (ta[2] + tb[2]) / A.dl;
        if (AXIS == 0)
        {
            double tauxx = mu * (vx_long - vy_tran);
            double tauxy = mu * (vy_long + vx_tran);
            F[1] = F[1] + -tauxx;
            F[2] = F[2] + -tauxy;
        }
        else
        {
            double tauyx = mu * (vy_tran + vx_long);
            double tauyy = -mu * (vx_tran - vy_long);
            F[1] = F[1] + -tauyx;
            F[2] = F[2] + -tauyy;
        }
    }
}

// FP32 form; the slopes ga, gb, ta, tb are doubled (vplm2).
template<int AXIS, typename T>
__device__ inline void face_flux_f(const T pa[3], const T pb[3], const T ga[3], const T gb[3], const T ta[3],
                                   const T tb[3], T x, T y, const FloatConsts& F, T out[3])
{
    T L[3], Rr[3];
    for (int k = 0; k < 3; ++k)
    {
        L[k] = vfma(bc<T>(0.25f), ga[k], pa[k]);
        Rr[k] = vfma(bc<T>(-0.25f), gb[k], pb[k]);
    }
    // sound_speed_squared at the face: -phi/M^2 with phi = -1/sqrt(r^2 + rs^2)
    const T rinv = vrsqrt(vfma(x, x, vfma(y, y, bc<T>(F.rs2))));
    const T cs2 = vmul(rinv, bc<T>(F.inv_mach2));
    const T cs = vsqrt(cs2);
    const T vl = AXIS == 0 ? L[1] : L[2];
    const T vr = AXIS == 0 ? Rr[1] : Rr[2];
    const T ul[3] = {L[0], vmul(L[0], L[1]), vmul(L[0], L[2])};
    const T ur[3] = {Rr[0], vmul(Rr[0], Rr[1]), vmul(Rr[0], Rr[2])};
    const T ap = vmax(bc<T>(0.0f), vadd(vmax(vl, vr), cs));
    const T am = vmin(bc<T>(0.0f), vsub(vmin(vl, vr), cs));
    // HLLE: (ap fl - am fr - (ul - ur) ap am) / (ap - am) = a fl + b fr + c (ur - ul)
    // with fl = vl ul + cs2 Sigma_l n, fr = vr ur + cs2 Sigma_r n, regrouped as
    // (a vl - c) ul + (b vr + c) ur + (a Sigma_l + b Sigma_r) cs2 n
    const T inv = vrcp(vsub(ap, am));
    const T ca = vmul(ap, inv), cb = vmul(vneg(am), inv), cc = vmul(vmul(ap, am), inv);
    const T wl = vfma(ca, vl, vneg(cc)), wr = vfma(cb, vr, cc);
    const T pn = vmul(vfma(ca, L[0], vmul(cb, Rr[0])), cs2);
    out[0] = vfma(wl, ul[0], vmul(wr, ur[0]));
    out[1] = AXIS == 0 ? vfma(wl, ul[1], vfma(wr, ur[1], pn)) : vfma(wl, ul[1], vmul(wr, ur[1]));
    out[2] = AXIS == 0 ? vfma(wl, ul[2], vmul(wr, ur[2])) : vfma(wl, ul[2], vfma(wr, ur[2], pn));
    if (F.half_nu != 0.0f)
    {
        // mu = nu (Sigma_l + Sigma_r) / 2 carries the 1/(4 dl) of the averaged doubled slopes
        const T mu = vmul(vadd(Rr[0], L[0]), bc<T>(F.visc_mu));
        const T nmu = vneg(mu);
        const T vx_long = vadd(ga[1], gb[1]);
        const T vy_long = vadd(ga[2], gb[2]);
        const T vx_tran = vadd(ta[1], tb[1]);
        const T vy_tran = vadd(ta[2], tb[2]);
        if (AXIS == 0)
        {
            out[1] = vfma(nmu, vsub(vx_long, vy_tran), out[1]);
            out[2] = vfma(nmu, vadd(vy_long, vx_tran), out[2]);
        }
        else
        {
            out[1] = vfma(nmu, vadd(vy_tran, vx_long), out[1]);
            out[2] = vfma(mu, vsub(vx_tran, vy_long), out[2]);
        }
    }
}

template<int AXIS>
__device__ inline void face_flux(const float pa[3], const float pb[3], const float ga[3], const float gb[3],
                                 const float ta[3], const float tb[3], float x, float y,
                                 const Args& A, float F[3])
{
    face_flux_f<AXIS, float>(pa, pb, ga, gb, ta, tb, x, y, A.f, F);
}

// ------------------------------------------------------------- mixed cell update
// Stage increment du = dt * L(u) of one cell (or a pair) in FP32: flux
// divergence, gravity of both point masses, sinks, rotating-frame terms and
// the outer buffer (problems/minidisk_scheme.cpp:337-352). uc returns the
// FP32 conserved state the increment was computed from, spot returns
// sqrt(1/sqrt(r^2 + rs^2)), the cell-centre sound speed times M.
__device__ __forceinline__ void diag_add(float& a, float v) { a += v; }
__device__ __forceinline__ void diag_add(float& a, float2 v) { a += v.x + v.y; }

// True where the calling lanes' q1 and q2 (each column of a pair) are all
// at least q_far.
__device__ __forceinline__ bool all_beyond(float q1, float q2, float q_far)
{
    return __all_sync(__activemask(), q1 >= q_far && q2 >= q_far);
}
__device__ __forceinline__ bool all_beyond(float2 q1, float2 q2, float q_far)
{
    return __all_sync(__activemask(), q1.x >= q_far && q1.y >= q_far && q2.x >= q_far && q2.y >= q_far);
}

template<typename T, bool DIAG = false>
__device__ inline void cell_increment(const FloatConsts& F, T x, T y, const T pc[3], const T dfx[3], const T dfy[3],
                                      const float bf[6], float dtf, T du[3], T uc[3], T& spot, float* acc = nullptr)
{
    uc[0] = pc[0];
    uc[1] = vmul(pc[0], pc[1]);
    uc[2] = vmul(pc[0], pc[2]);
    const T dx1 = vsub(x, bc<T>(bf[1])), dy1 = vsub(y, bc<T>(bf[2]));
    const T dx2 = vsub(x, bc<T>(bf[4])), dy2 = vsub(y, bc<T>(bf[5]));
    const T q1 = vfma(dx1, dx1, vmul(dy1, dy1)), q2 = vfma(dx2, dx2, vmul(dy2, dy2));
    const T i1 = vrsqrt(vadd(q1, bc<T>(F.rs2))), i2 = vrsqrt(vadd(q2, bc<T>(F.rs2)));
    const T g1 = vmul(vmul(vmul(bc<T>(-bf[0]), i1), i1), i1);
    const T g2 = vmul(vmul(vmul(bc<T>(-bf[3]), i2), i2), i2);
    // sinks: sink_rate exp(-r^6 / s^6) as sink_rate 2^(q^3 sink_ex2), q = r^2.
    // Where every cell of the warp lies at q >= sink_far from both bodies
    // (nearly all of the mesh), the flushed 2^(...) is exactly zero for all
    // of them, and the warp skips it.
    T e1 = bc<T>(0.0f), e2 = bc<T>(0.0f), srs = bc<T>(0.0f);
    if (!all_beyond(q1, q2, F.sink_far))
    {
        e1 = vex2(vmul(vmul(q1, q1), vmul(q1, bc<T>(F.sink_ex2))));
        e2 = vex2(vmul(vmul(q2, q2), vmul(q2, bc<T>(F.sink_ex2))));
        srs = vmul(bc<T>(F.sink_rate), vadd(e1, e2));
    }
    const T r2 = vfma(x, x, vmul(y, y));
    const T rinv = vrsqrt(r2);
    const T rr = vmul(r2, rinv);
    // 0.5*rate*(1 + tanh(z)) written as rate / (1 + exp(-2z))
    const T br = vmul(bc<T>(F.buffer_rate),
                      vrcp(vadd(bc<T>(1.0f), vex2(vmul(vsub(rr, bc<T>(F.R)), bc<T>(F.buffer_ex2))))));
    spot = vsqrt(vrsqrt(vadd(r2, bc<T>(F.rs2))));
    // Keplerian velocity of the buffer target, over r: (sqrt(pot) - omega r) / r
    const T vpr = vmul(vfma(bc<T>(-F.omega), rr, spot), rinv);
    const T ui1 = vmul(vneg(vpr), y), ui2 = vmul(vpr, x);
    T ax = vfma(g2, dx2, vmul(g1, dx1));
    ax = vfma(bc<T>(F.omega2), x, ax);
    ax = vfma(bc<T>(F.two_omega), pc[2], ax);
    T ay = vfma(g2, dy2, vmul(g1, dy1));
    ay = vfma(bc<T>(F.omega2), y, ay);
    ay = vfma(bc<T>(-F.two_omega), pc[1], ay);
    if constexpr (DIAG)
    {
        // the rate-vector sums of this cell (times the cell area on the flush)
        const T sr1 = vmul(bc<T>(F.sink_rate), e1), sr2 = vmul(bc<T>(F.sink_rate), e2);
        const T sg1 = vmul(pc[0], g1), sg2 = vmul(pc[0], g2);
        diag_add(acc[0], vmul(pc[0], sr1));
        diag_add(acc[1], vmul(pc[0], sr2));
        diag_add(acc[2], vmul(uc[1], sr1));
        diag_add(acc[3], vmul(uc[2], sr1));
        diag_add(acc[4], vmul(uc[1], sr2));
        diag_add(acc[5], vmul(uc[2], sr2));
        diag_add(acc[6], vneg(vmul(sg1, dx1)));
        diag_add(acc[7], vneg(vmul(sg1, dy1)));
        diag_add(acc[8], vneg(vmul(sg2, dx2)));
        diag_add(acc[9], vneg(vmul(sg2, dy2)));
        diag_add(acc[10], vmul(vsub(bc<T>(1.0f), pc[0]), br));
        diag_add(acc[11], pc[0]);
        diag_add(acc[12], vsub(vmul(x, uc[2]), vmul(y, uc[1])));
    }
    // buffer toward ui = (1, ui1, ui2) and sinks: (ui - uc) br - uc srs = ui br - uc (br + srs)
    const T sb = vadd(br, srs);
    T src[3];
    src[0] = vfma(vneg(uc[0]), sb, br);
    src[1] = vfma(pc[0], ax, vfma(ui1, br, vneg(vmul(uc[1], sb))));
    src[2] = vfma(pc[0], ay, vfma(ui2, br, vneg(vmul(uc[2], sb))));
    for (int k = 0; k < 3; ++k)
        du[k] = vmul(bc<T>(dtf), vfma(vadd(dfx[k], dfy[k]), bc<T>(-F.inv_dl), src[k]));
}

// Operands of one cell's (or one pair's) FP64 store, loaded ahead of the
// flux work so that their latency hides behind it: the stage-input state and,
// in stage 2 of RK2, the stage-1 increment.
template<typename T> struct CellIn;
template<> struct CellIn<float> { double u[3]; float d[3]; };
template<> struct CellIn<float2> { double2 u[3]; float2 d[3]; };

// Stage 1 of mixed RK2 stores only the FP32 increment; every other mixed
// stage writes an FP64 state.
template<int KIND>
__device__ inline bool writes_state(const Args& A) { return KIND != K_MIXD && !(KIND == K_MIX1 && A.d_out); }

template<int KIND>
__device__ inline void load_cell_in(const Args& A, size_t idx, size_t NN, CellIn<float>& c)
{
    if (!writes_state<KIND>(A)) return;
    for (int k = 0; k < 3; ++k) c.u[k] = __ldg(A.u_in + k * NN + idx);
    if (KIND == K_MIX2)
        for (int k = 0; k < 3; ++k) c.d[k] = __ldg(A.d1 + k * NN + idx);
}

template<int KIND>
__device__ inline void load_cell_in(const Args& A, size_t idx, size_t NN, CellIn<float2>& c)
{
    if (!writes_state<KIND>(A)) return;
    for (int k = 0; k < 3; ++k) c.u[k] = __ldg(reinterpret_cast<const double2*>(A.u_in + k * NN + idx));
    if (KIND == K_MIX2)
        for (int k = 0; k < 3; ++k) c.d[k] = __ldg(reinterpret_cast<const float2*>(A.d1 + k * NN + idx));
}

// The mixed path's CFL reduction: the FP32 wavespeed's bits in the high word
// and the cell index in the low word. The maximum key names the fastest cell
// (ties go to the larger index, whatever the launch shape); the clock then
// evaluates that cell's wavespeed in FP64 from the FP64 state, so the CFL dt
// is an FP64 quantity as in the FP64 path.
__device__ __forceinline__ unsigned long long speed_key(float v, size_t idx)
{
    return (static_cast<unsigned long long>(__float_as_uint(v)) << 32) | static_cast<unsigned>(idx);
}

__device__ __forceinline__ unsigned long long key_max(unsigned long long a, unsigned long long b) { return a > b ? a : b; }

// A thread's running maximum of speed keys, for cells visited in any order.
struct KeyMax
{
    unsigned long long k = 0ull;
    __device__ __forceinline__ void take(float v, size_t idx) { k = key_max(k, speed_key(v, idx)); }
    __device__ __forceinline__ unsigned long long key() const { return k; }
};

// The same maximum for a sweep lane, whose cells arrive in increasing index
// order: the wavespeed bits and the index of the fastest so far, kept apart
// (one unsigned comparison per cell instead of a 64-bit key and its
// comparison). >= moves ties to the later, larger index, so key() equals
// KeyMax's key over the same cells.
struct LaneMax
{
    unsigned bits = 0u, idx = 0u;
    __device__ __forceinline__ void take(float v, size_t i)
    {
        const unsigned b = __float_as_uint(v);
        if (b >= bits)
        {
            bits = b;
            idx = unsigned(i);
        }
    }
    __device__ __forceinline__ unsigned long long key() const
    {
        return (static_cast<unsigned long long>(bits) << 32) | idx;
    }
};

// The end of a warp's CFL reduction: the key, or the FP32 maximum as double
// bits where the caller asked for the wavespeed itself.
__device__ inline void flush_speed_key(const Args& A, unsigned long long key)
{
    for (int o = 16; o > 0; o >>= 1) key = key_max(key, __shfl_xor_sync(0xffffffffu, key, o));
    if ((threadIdx.x & 31) == 0)
    {
        const float v = __uint_as_float(unsigned(key >> 32));
        atomicMax(A.amax, A.amax_key ? key : (unsigned long long)__double_as_longlong(double(v)));
    }
}

// Fastest wavespeed max(|vx|, |vy|) + cs (iso2d::fastest_wavespeed,
// physics_iso2d.hpp:108-116) of an FP32 conserved state at a cell whose
// sqrt(1/sqrt(r^2 + rs^2)) is spot. max(|m1|, |m2|) / s equals the larger of
// the two velocities exactly (rounding is monotonic).
__device__ inline float wavespeed_f(const FloatConsts& F, float s, float m1, float m2, float spot)
{
    return vfma(fmaxf(fabsf(m1), fabsf(m2)), rcp_fast(s), vmul(spot, F.inv_mach));
}

// One cell's stage result: the FP32 increment (stage 1 of mixed RK2), or the
// FP64 state u_in + du (with the RK2 average of the two increments in stage
// 2). The CFL wavespeed of the new state is taken from its FP32 image: the
// stage input plus du (RK1), or u0 + (d1 + du)/2 = u1 + (du - d1)/2 (RK2).
template<int KIND, bool DIAG = false, typename Max>
__device__ inline void mixed_cell(const Args& A, float x, float y, const float pc[3], const float dfx[3],
                                  const float dfy[3], const float bf[6], float dtf, size_t idx, size_t NN,
                                  const CellIn<float>& in, Max& local_max, float* acc = nullptr)
{
    float du[3], uc[3], spot;
    cell_increment<float, DIAG>(A.f, x, y, pc, dfx, dfy, bf, dtf, du, uc, spot, acc);
    if (!writes_state<KIND>(A))
    {
        for (int k = 0; k < 3; ++k) A.d_out[k * NN + idx] = du[k];
        return;
    }
    float of[3];
    for (int k = 0; k < 3; ++k)
    {
        const float inc = KIND == K_MIX2 ? vadd(in.d[k], du[k]) : du[k];
        A.u_out[k * NN + idx] = __fma_rn(f2d_sum(inc), KIND == K_MIX2 ? 0.5 : 1.0, in.u[k]);
        of[k] = KIND == K_MIX2 ? vfma(vsub(du[k], in.d[k]), 0.5f, uc[k]) : vadd(uc[k], du[k]);
    }
    if (A.amax) local_max.take(wavespeed_f(A.f, of[0], of[1], of[2], spot), idx);
}

// The pair form: columns idx and idx + 1 of one row (idx even).
template<int KIND, bool DIAG = false>
__device__ inline void mixed_cell2(const Args& A, float2 x, float2 y, const float2 pc[3], const float2 dfx[3],
                                   const float2 dfy[3], const float bf[6], float dtf, size_t idx, size_t NN,
                                   const CellIn<float2>& in, LaneMax& local_max, float* acc = nullptr)
{
    float2 du[3], uc[3], spot;
    cell_increment<float2, DIAG>(A.f, x, y, pc, dfx, dfy, bf, dtf, du, uc, spot, acc);
    if (!writes_state<KIND>(A))
    {
        for (int k = 0; k < 3; ++k) *reinterpret_cast<float2*>(A.d_out + k * NN + idx) = du[k];
        return;
    }
    float2 of[3];
    for (int k = 0; k < 3; ++k)
    {
        // RK2: u0 + (d1 + d2)/2, the halving exact inside the FP64 fma; RK1: u + du
        const float2 inc = KIND == K_MIX2 ? vadd(in.d[k], du[k]) : du[k];
        const double h = KIND == K_MIX2 ? 0.5 : 1.0;
        *reinterpret_cast<double2*>(A.u_out + k * NN + idx) = make_double2(__fma_rn(f2d_sum(inc.x), h, in.u[k].x),
                                                                           __fma_rn(f2d_sum(inc.y), h, in.u[k].y));
        of[k] = KIND == K_MIX2 ? vfma(vsub(du[k], in.d[k]), bc<float2>(0.5f), uc[k]) : vadd(uc[k], du[k]);
    }
    if (A.amax)
    {
        local_max.take(wavespeed_f(A.f, of[0].x, of[1].x, of[2].x, spot.x), idx);
        local_max.take(wavespeed_f(A.f, of[0].y, of[1].y, of[2].y, spot.y), idx + 1);
    }
}

// A warp's diagnostic sums into the stage's rate row: FP32 per lane, a
// shuffle reduction, then FP64 atomics scaled by the cell area.
__device__ inline void diag_flush(const Args& A, const float* acc)
{
    const double da = A.dl * A.dl;
    for (int k = 0; k < DIAG_SUMS; ++k)
    {
        float v = acc[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(A.diag + k, double(v) * da);
    }
}

// ------------------------------------------------------------- warp-strip sweep (mixed path)
// One warp updates a strip of SW_COLS columns (its 32 lanes hold columns
// j0-2 .. j0+29: two halo columns each side) over A.sweep_rows rows, marching
// along x. A three-row window of primitives, the x and y slopes of two rows
// and the previous x-face flux stay in registers; y neighbours come from warp
// shuffles. Every x face and y face of the strip is computed once, with no
// shared memory and no barrier. Requires N >= 64 (halo wrap by one period).
constexpr int SW_COLS = 28, SW_WARPS = 4;

__device__ inline int wrap1(int g, int N) { return g < 0 ? g + N : (g >= N ? g - N : g); }

// One row of this lane's column, raw: FP64 state (+ FP32 stage-1 increment).
struct RawRow
{
    double u[3];
    float d[3];
};

template<int KIND>
__device__ inline void sweep_fetch(const Args& A, int row, int jg, size_t NN, RawRow& r)
{
    const size_t idx = size_t(wrap1(row, A.N)) * A.N + jg;
    for (int k = 0; k < 3; ++k) r.u[k] = __ldg(A.u_in + k * NN + idx);
    if (KIND == K_MIX2)
        for (int k = 0; k < 3; ++k) r.d[k] = __ldg(A.d1 + k * NN + idx);
}

template<int KIND>
__device__ inline void sweep_prim(const RawRow& r, float p[3])
{
    float s = d2f(r.u[0]), m1 = d2f(r.u[1]), m2 = d2f(r.u[2]);
    if (KIND == K_MIX2)
    {
        s = vadd(s, r.d[0]);
        m1 = vadd(m1, r.d[1]);
        m2 = vadd(m2, r.d[2]);
    }
    const float inv = vrcp(s);
    p[0] = s;
    p[1] = div_corrected(m1, s, inv);
    p[2] = div_corrected(m2, s, inv);
}

__device__ inline void slope_y(const float p[3], float two_theta, float g[3])
{
    for (int k = 0; k < 3; ++k)
    {
        float l = __shfl_up_sync(0xffffffffu, p[k], 1);
        float r = __shfl_down_sync(0xffffffffu, p[k], 1);
        g[k] = vplm2(l, p[k], r, two_theta);
    }
}

// Rows [i0, i1) of column strip sy of the mesh A describes: the body of a
// sweep warp. Called with a warp-uniform (i0, i1, sy).
template<int KIND, bool DIAG = false>
__device__ __forceinline__ void sweep_strip(const Args& A, int i0, int i1, int sy)
{
    const int lane = threadIdx.x & 31;
    const int N = A.N;
    const int jcol = sy * SW_COLS - 2 + lane;  // unwrapped column of this lane
    const int jg = wrap1(jcol, N);
    const bool interior = lane >= 2 && lane < 2 + SW_COLS && jcol < N;
    const size_t NN = size_t(N) * N;
    const FloatConsts& F = A.f;
    const float theta = F.two_theta;   // doubled slopes (vplm2)

    float bf[6];
    double dt;
    if (A.clock)
    {
        dt = A.clock->dt;
        for (int k = 0; k < 6; ++k) bf[k] = d2f(A.clock->binary[A.stage][k]);
    }
    else
    {
        dt = A.dt;
        for (int k = 0; k < 6; ++k) bf[k] = d2f(A.bin[k]);
    }
    const float dtf = d2f(dt);
    const float yc = fmaf(float(jcol) + 0.5f, F.dl, -F.R);   // this lane's cell centre
    const float yv = fmaf(float(jcol), F.dl, -F.R);          // face between lanes l-1 and l

    // prologue: rows i0-2 .. i0+1, and the fetch of row i0+2
    float pm2[3], pm1[3], p0[3], p1[3];
    RawRow raw;
    sweep_fetch<KIND>(A, i0 - 2, jg, NN, raw);
    sweep_prim<KIND>(raw, pm2);
    sweep_fetch<KIND>(A, i0 - 1, jg, NN, raw);
    sweep_prim<KIND>(raw, pm1);
    sweep_fetch<KIND>(A, i0, jg, NN, raw);
    sweep_prim<KIND>(raw, p0);
    sweep_fetch<KIND>(A, i0 + 1, jg, NN, raw);
    sweep_prim<KIND>(raw, p1);
    sweep_fetch<KIND>(A, i0 + 2, jg, NN, raw);
    float gxm1[3], gx0[3], gym1[3], gy0[3], fxm[3];
    for (int k = 0; k < 3; ++k)
    {
        gxm1[k] = vplm2(pm2[k], pm1[k], p0[k], theta);
        gx0[k] = vplm2(pm1[k], p0[k], p1[k], theta);
    }
    slope_y(pm1, theta, gym1);
    slope_y(p0, theta, gy0);
    face_flux<0>(pm1, p0, gxm1, gx0, gym1, gy0, fmaf(float(i0), F.dl, -F.R), yc, A, fxm);

    LaneMax local_max;
    float acc[DIAG ? DIAG_SUMS : 1] = {};
    for (int i = i0; i < i1; ++i)
    {
        float p2[3], gx1[3], gy1[3], fxp[3];
        sweep_prim<KIND>(raw, p2);                       // row i+2, fetched last iteration
        sweep_fetch<KIND>(A, i + 3, jg, NN, raw);        // in flight during this row
        CellIn<float> cin;
        if (interior) load_cell_in<KIND>(A, size_t(i) * N + jg, NN, cin);
        for (int k = 0; k < 3; ++k) gx1[k] = vplm2(p0[k], p1[k], p2[k], theta);
        slope_y(p1, theta, gy1);
        face_flux<0>(p0, p1, gx0, gx1, gy0, gy1, fmaf(float(i + 1), F.dl, -F.R), yc, A, fxp);

        // y face on this lane's left side, from lane l-1 (row i)
        float pl[3], gl[3], tl[3], fy[3];
        for (int k = 0; k < 3; ++k)
        {
            pl[k] = __shfl_up_sync(0xffffffffu, p0[k], 1);
            gl[k] = __shfl_up_sync(0xffffffffu, gy0[k], 1);
            tl[k] = __shfl_up_sync(0xffffffffu, gx0[k], 1);
        }
        const float xc = fmaf(float(i) + 0.5f, F.dl, -F.R);
        face_flux<1>(pl, p0, gl, gy0, tl, gx0, xc, yv, A, fy);
        float dfx[3], dfy[3];
        for (int k = 0; k < 3; ++k)
        {
            dfy[k] = vsub(__shfl_down_sync(0xffffffffu, fy[k], 1), fy[k]);
            dfx[k] = vsub(fxp[k], fxm[k]);
        }
        if (interior)
            mixed_cell<KIND, DIAG>(A, xc, yc, p0, dfx, dfy, bf, dtf, size_t(i) * N + jg, NN, cin, local_max, acc);

        for (int k = 0; k < 3; ++k)
        {
            p0[k] = p1[k];
            p1[k] = p2[k];
            gx0[k] = gx1[k];
            gy0[k] = gy1[k];
            fxm[k] = fxp[k];
        }
    }
    if constexpr (DIAG) diag_flush(A, acc);
    if (A.amax) flush_speed_key(A, local_max.key());
}

// ------------------------------------------------------------- two-column sweep
// Thread coarsening of the sweep: lane l holds the column pair
// (j0 - 2 + 2l, j0 - 1 + 2l), so a warp covers 64 columns of which 60 are
// interior (the 1-column sweep keeps 28 of 32): half the y-direction
// shuffles per cell, a smaller share of halo lanes, and double2 / float2
// loads and stores. The arithmetic is that of the 1-column sweep, so the
// results are bit-identical. Requires an even N >= 64 and 16-byte aligned
// state (8-byte aligned increments).
constexpr int SW2_COLS = 60;

struct RawRow2
{
    double2 u[3];
    float2 d[3];
};

template<int KIND>
__device__ inline void sweep2_fetch(const Args& A, int row, int jg, size_t NN, RawRow2& r)
{
    const size_t idx = size_t(wrap1(row, A.N)) * A.N + jg;
    for (int k = 0; k < 3; ++k) r.u[k] = __ldg(reinterpret_cast<const double2*>(A.u_in + k * NN + idx));
    if (KIND == K_MIX2)
        for (int k = 0; k < 3; ++k) r.d[k] = __ldg(reinterpret_cast<const float2*>(A.d1 + k * NN + idx));
}

template<int KIND>
__device__ inline void sweep2_prim(const RawRow2& r, float2 p[3])
{
    float2 s = make_float2(d2f(r.u[0].x), d2f(r.u[0].y));
    float2 m1 = make_float2(d2f(r.u[1].x), d2f(r.u[1].y));
    float2 m2 = make_float2(d2f(r.u[2].x), d2f(r.u[2].y));
    if (KIND == K_MIX2)
    {
        s = vadd(s, r.d[0]);
        m1 = vadd(m1, r.d[1]);
        m2 = vadd(m2, r.d[2]);
    }
    const float2 inv = vrcp(s);
    p[0] = s;
    p[1] = make_float2(div_corrected(m1.x, s.x, inv.x), div_corrected(m1.y, s.y, inv.y));
    p[2] = make_float2(div_corrected(m2.x, s.x, inv.x), div_corrected(m2.y, s.y, inv.y));
}

// Per-warp ring of five rows in shared memory, filled by per-lane
// asynchronous copies (cp.async): the row being recovered (i+2), two rows in
// flight (i+3, i+4), and the rows whose stage results are written (i, i+1),
// which then need no second global load. Each lane copies and reads only its
// own two columns, so no lane waits on another. Ring slot of row r >= -2:
// (r + 5) mod 5.
constexpr int RING_ROWS = 5;
constexpr int RING_U_BYTES = RING_ROWS * 3 * 32 * 16;     // double2 per lane and component
constexpr int RING_D_BYTES = RING_ROWS * 3 * 32 * 8;      // float2 per lane and component
constexpr int RING_WARP_BYTES = RING_U_BYTES + RING_D_BYTES;

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

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ int ring_slot(int row) { return (row + RING_ROWS) % RING_ROWS; }

struct Ring2
{
    double2* u;    // [row slot][component][lane]
    float2* d;
};

template<int KIND>
__device__ inline void ring2_fetch(const Args& A, const Ring2& R, int row, int jg, size_t NN, int lane,
                                   int slot = -1)
{
    if (slot < 0) slot = ring_slot(row);
    const size_t idx = size_t(wrap1(row, A.N)) * A.N + jg;
    for (int k = 0; k < 3; ++k) cp_async16(&R.u[(slot * 3 + k) * 32 + lane], A.u_in + k * NN + idx);
    if (KIND == K_MIX2)
        for (int k = 0; k < 3; ++k) cp_async8(&R.d[(slot * 3 + k) * 32 + lane], A.d1 + k * NN + idx);
    cp_async_commit();
}

template<int KIND>
__device__ inline void ring2_row(const Ring2& R, int row, int lane, RawRow2& r, int slot = -1)
{
    if (slot < 0) slot = ring_slot(row);
    for (int k = 0; k < 3; ++k) r.u[k] = R.u[(slot * 3 + k) * 32 + lane];
    if (KIND == K_MIX2)
        for (int k = 0; k < 3; ++k) r.d[k] = R.d[(slot * 3 + k) * 32 + lane];
}

// y slopes of both columns: the left neighbour of the first column is lane
// l-1's second column (returned in left, which the row's y faces reuse), the
// right neighbour of the second is lane l+1's first.
__device__ inline void slope_y2(const float2 p[3], float two_theta, float2 g[3], float left[3])
{
    for (int k = 0; k < 3; ++k)
    {
        left[k] = __shfl_up_sync(0xffffffffu, p[k].y, 1);
        const float r = __shfl_down_sync(0xffffffffu, p[k].x, 1);
        g[k] = vplm2(make_float2(left[k], p[k].x), p[k], make_float2(p[k].y, r), two_theta);
    }
}

// The same five-row ring filled by the tensor memory accelerator: for each
// row one elected lane issues one bulk tensor copy of the strip's 64 columns
// of the three FP64 components (box 64 x 1 x 3 of the [3][N][N] state), and
// in stage 2 one of the FP32 increment (box 68 x 1 x 3 from column j0 - 4, so
// that the box starts on a 16-byte boundary), completing on the slot's
// mbarrier. The lanes wait on the barrier (a bounded wait) and read their
// two columns as from the per-lane ring. Strips whose 64 columns wrap across
// the periodic seam (the first and the last) keep the per-lane ring: a box
// cannot wrap.
constexpr int TRING_U_SLOT = 3 * 64 * 8;                     // 1536 B per slot: 3 components x 64 doubles
constexpr int TRING_D_COLS = 68;                             // floats per component row of the increment box
constexpr int TRING_D_SLOT = 896;                            // 3 x 68 floats (816 B), padded to 128-byte slots
constexpr int TRING_BAR_OFFSET = RING_ROWS * (TRING_U_SLOT + TRING_D_SLOT);
constexpr int TRING_WARP_BYTES = TRING_BAR_OFFSET + 128;     // + five mbarriers: 12288 B per warp
static_assert(TRING_WARP_BYTES >= RING_WARP_BYTES, "the per-lane ring must fit in a TMA ring's region");
static_assert(TRING_U_SLOT % 128 == 0 && TRING_D_SLOT % 128 == 0 && TRING_WARP_BYTES % 128 == 0,
              "bulk tensor copies land on 128-byte boundaries");

struct RingT
{
    unsigned char* base;       // 128-byte aligned: u slots, then d slots, then the barriers
    const CUtensorMap* umap;   // [3][N][N] FP64 state, box 64 x 1 x 3
    const CUtensorMap* dmap;   // [3][N][N] FP32 increment, box 68 x 1 x 3 (stage 2)
    int xu, xd;                // first column of the boxes: j0 - 2, j0 - 4 (both 16-byte aligned)
    int row0;                  // first row fetched (i0 - 2); fetches follow in row order
    int last_fetch, last_wait; // highest row fetched / waited for
    bool broken;               // a copy did not complete in time: rows come from global memory from then on
};

// a strip whose 64 columns j0 - 2 .. j0 + 61 (and the increment box's 68
// from j0 - 4) lie inside the mesh
__host__ __device__ inline bool tma_strip(int sy, int N) { return sy >= 1 && sy * SW2_COLS + 64 <= N; }

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }
__device__ __forceinline__ uint32_t tring_bar(const RingT& R, int slot)
{
    return smem_u32(R.base + TRING_BAR_OFFSET + 8 * slot);
}

__device__ inline void tring_init(RingT& R, int lane)
{
    if (lane == 0)
    {
        for (int s = 0; s < RING_ROWS; ++s)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(tring_bar(R, s)), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
}

// Row `row` into its slot. Every lane has finished reading the row the slot
// held before (its last read was an iteration ago); the proxy fence orders
// those reads before the copy's writes.
template<int KIND>
__device__ inline void tring_fetch(const Args& A, RingT& R, int row, int lane)
{
    if (R.broken) return;
    const int slot = ring_slot(row);
    __syncwarp();
    if (lane == 0)
    {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const uint32_t bar = tring_bar(R, slot);
        const uint32_t bytes = TRING_U_SLOT + (KIND == K_MIX2 ? 3 * TRING_D_COLS * 4 : 0);
        const int r = wrap1(row, A.N);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(bar), "r"(bytes) : "memory");
        asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
                     " [%0], [%1, {%2, %3, %4}], [%5];"
                     :: "r"(smem_u32(R.base + slot * TRING_U_SLOT)), "l"(reinterpret_cast<uint64_t>(R.umap)),
                        "r"(R.xu), "r"(r), "r"(0), "r"(bar)
                     : "memory");
        if (KIND == K_MIX2)
            asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
                         " [%0], [%1, {%2, %3, %4}], [%5];"
                         :: "r"(smem_u32(R.base + RING_ROWS * TRING_U_SLOT + slot * TRING_D_SLOT)),
                            "l"(reinterpret_cast<uint64_t>(R.dmap)), "r"(R.xd), "r"(r), "r"(0), "r"(bar)
                         : "memory");
    }
    R.last_fetch = row;
}

// Bounded wait for row `row` (the phase of its slot's barrier that its fetch
// completes: the k-th fetch into a slot completes phase k, and with fetches
// in row order k = (row - row0) / 5). True where every lane saw it complete.
__device__ inline bool tring_wait(const RingT& R, int row)
{
    const uint32_t bar = tring_bar(R, ring_slot(row));
    const uint32_t parity = uint32_t((row - R.row0) / RING_ROWS) & 1u;
    uint32_t done = 0;
    for (int it = 0; it < (1 << 20) && !done; ++it)
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}" : "=r"(done) : "r"(bar), "r"(parity) : "memory");
    return __all_sync(0xffffffffu, done != 0);
}

// This lane's two columns of row `row` from its slot (the row has arrived)
template<int KIND>
__device__ inline void tring_row(const RingT& R, int row, int lane, RawRow2& r)
{
    const int slot = ring_slot(row);
    const double2* u = reinterpret_cast<const double2*>(R.base + slot * TRING_U_SLOT);
    for (int k = 0; k < 3; ++k) r.u[k] = u[k * 32 + lane];
    if (KIND == K_MIX2)
    {
        // float index k * 68 + (2 lane + 2): the box starts two columns left of the strip
        const float2* d = reinterpret_cast<const float2*>(R.base + RING_ROWS * TRING_U_SLOT + slot * TRING_D_SLOT);
        for (int k = 0; k < 3; ++k) r.d[k] = d[k * (TRING_D_COLS / 2) + lane + 1];
    }
}

// Row `row` for the recovery: from the ring once it has arrived, else (a
// timed-out copy) from global memory, for this row and every later one.
template<int KIND>
__device__ inline void tring_get(const Args& A, RingT& R, int row, int jg, size_t NN, int lane, RawRow2& r)
{
    if (!R.broken)
    {
        if (tring_wait(R, row))
        {
            R.last_wait = row;
            tring_row<KIND>(R, row, lane, r);
            return;
        }
        R.broken = true;
    }
    sweep2_fetch<KIND>(A, row, jg, NN, r);
}

// Before the warp leaves: wait (bounded) for the rows fetched but not
// waited for, so that no copy lands in shared memory after the warp is gone.
__device__ inline void tring_drain(const RingT& R)
{
    for (int row = R.last_wait + 1; row <= R.last_fetch; ++row) tring_wait(R, row);
}

template<int KIND, bool DIAG = false, int RING = 0>
__device__ __forceinline__ void sweep_strip2(const Args& A, int i0, int i1, int sy, Ring2 ring = Ring2{},
                                             RingT* tma = nullptr)
{
    const int lane = threadIdx.x & 31;
    const int N = A.N;
    const int jcol = sy * SW2_COLS - 2 + 2 * lane;    // unwrapped first column of this lane's pair
    const int jg = wrap1(jcol, N);                      // N even: the pair stays adjacent after the wrap
    const bool interior = lane >= 1 && lane < 1 + SW2_COLS / 2 && jcol < N;
    const size_t NN = size_t(N) * N;
    const FloatConsts& F = A.f;
    const float theta = F.two_theta;   // doubled slopes (vplm2)

    float bf[6];
    double dt;
    if (A.clock)
    {
        dt = A.clock->dt;
        for (int k = 0; k < 6; ++k) bf[k] = d2f(A.clock->binary[A.stage][k]);
    }
    else
    {
        dt = A.dt;
        for (int k = 0; k < 6; ++k) bf[k] = d2f(A.bin[k]);
    }
    const float dtf = d2f(dt);
    // cell centres of the pair, and the faces on the left of each column
    const float2 yc = make_float2(fmaf(float(jcol) + 0.5f, F.dl, -F.R), fmaf(float(jcol + 1) + 0.5f, F.dl, -F.R));
    const float2 yv = make_float2(fmaf(float(jcol), F.dl, -F.R), fmaf(float(jcol + 1), F.dl, -F.R));

    float2 pm2[3], pm1[3], p0[3], p1[3];
    RawRow2 raw;
    if constexpr (RING == 2)
    {
        RingT& T = *tma;
        T.row0 = i0 - 2;
        T.last_fetch = T.last_wait = i0 - 3;
        T.broken = false;
        tring_init(T, lane);
        for (int r = i0 - 2; r <= i0 + 1; ++r) tring_fetch<KIND>(A, T, r, lane);
        tring_get<KIND>(A, T, i0 - 2, jg, NN, lane, raw);
        sweep2_prim<KIND>(raw, pm2);
        tring_get<KIND>(A, T, i0 - 1, jg, NN, lane, raw);
        sweep2_prim<KIND>(raw, pm1);
        tring_get<KIND>(A, T, i0, jg, NN, lane, raw);
        sweep2_prim<KIND>(raw, p0);
        tring_get<KIND>(A, T, i0 + 1, jg, NN, lane, raw);
        sweep2_prim<KIND>(raw, p1);
        tring_fetch<KIND>(A, T, i0 + 2, lane);     // into the fifth, free slot
        tring_fetch<KIND>(A, T, i0 + 3, lane);     // into the slot of row i0 - 2
    }
    else if constexpr (RING == 1)
    {
        for (int r = i0 - 2; r <= i0 + 1; ++r) ring2_fetch<KIND>(A, ring, r, jg, NN, lane);
        cp_async_wait_all();
        ring2_row<KIND>(ring, i0 - 2, lane, raw);
        sweep2_prim<KIND>(raw, pm2);
        ring2_row<KIND>(ring, i0 - 1, lane, raw);
        sweep2_prim<KIND>(raw, pm1);
        ring2_row<KIND>(ring, i0, lane, raw);
        sweep2_prim<KIND>(raw, p0);
        ring2_row<KIND>(ring, i0 + 1, lane, raw);
        sweep2_prim<KIND>(raw, p1);
        ring2_fetch<KIND>(A, ring, i0 + 2, jg, NN, lane);     // into the fifth, free slot
        ring2_fetch<KIND>(A, ring, i0 + 3, jg, NN, lane);     // into the slot of row i0 - 2
    }
    else
    {
        sweep2_fetch<KIND>(A, i0 - 2, jg, NN, raw);
        sweep2_prim<KIND>(raw, pm2);
        sweep2_fetch<KIND>(A, i0 - 1, jg, NN, raw);
        sweep2_prim<KIND>(raw, pm1);
        sweep2_fetch<KIND>(A, i0, jg, NN, raw);
        sweep2_prim<KIND>(raw, p0);
        sweep2_fetch<KIND>(A, i0 + 1, jg, NN, raw);
        sweep2_prim<KIND>(raw, p1);
        sweep2_fetch<KIND>(A, i0 + 2, jg, NN, raw);
    }
    float2 gxm1[3], gx0[3], gym1[3], gy0[3], fxm[3];
    for (int k = 0; k < 3; ++k)
    {
        gxm1[k] = vplm2(pm2[k], pm1[k], p0[k], theta);
        gx0[k] = vplm2(pm1[k], p0[k], p1[k], theta);
    }
    float lm1[3], l0[3];
    slope_y2(pm1, theta, gym1, lm1);
    slope_y2(p0, theta, gy0, l0);
    face_flux_f<0, float2>(pm1, p0, gxm1, gx0, gym1, gy0, bc<float2>(fmaf(float(i0), F.dl, -F.R)), yc, F, fxm);

    LaneMax local_max;
    float acc[DIAG ? DIAG_SUMS : 1] = {};
    int slot0 = ring_slot(i0);                                // ring slot of row i, kept by increments
    for (int i = i0; i < i1; ++i)
    {
        float2 p2[3], gx1[3], gy1[3], fxp[3];
        CellIn<float2> cin;
        if constexpr (RING == 2)
        {
            tring_get<KIND>(A, *tma, i + 2, jg, NN, lane, raw);
            sweep2_prim<KIND>(raw, p2);
            tring_fetch<KIND>(A, *tma, i + 4, lane);              // into the slot of row i-1
        }
        else if constexpr (RING == 1)
        {
            const int slot2 = slot0 >= RING_ROWS - 2 ? slot0 + 2 - RING_ROWS : slot0 + 2;
            const int slot4 = slot0 == 0 ? RING_ROWS - 1 : slot0 - 1;
            cp_async_wait_one();                              // row i+2 (row i+3 may stay in flight)
            ring2_row<KIND>(ring, i + 2, lane, raw, slot2);
            sweep2_prim<KIND>(raw, p2);
            ring2_fetch<KIND>(A, ring, i + 4, jg, NN, lane, slot4);  // into the slot of row i-1
        }
        else
        {
            sweep2_prim<KIND>(raw, p2);                       // row i+2, fetched last iteration
            sweep2_fetch<KIND>(A, i + 3, jg, NN, raw);        // in flight during this row
            if (interior) load_cell_in<KIND>(A, size_t(i) * N + jg, NN, cin);
        }
        float l1[3];
        for (int k = 0; k < 3; ++k) gx1[k] = vplm2(p0[k], p1[k], p2[k], theta);
        slope_y2(p1, theta, gy1, l1);
        face_flux_f<0, float2>(p0, p1, gx0, gx1, gy0, gy1, bc<float2>(fmaf(float(i + 1), F.dl, -F.R)), yc, F, fxp);

        // y faces on the left of both columns (row i): the first from lane l-1's
        // second column (its primitives shuffled with the row's y slopes; the
        // density's transverse slope is not used)
        float2 pa[3], ga[3], ta[3], fy[3];
        for (int k = 0; k < 3; ++k)
        {
            pa[k] = make_float2(l0[k], p0[k].x);
            ga[k] = make_float2(__shfl_up_sync(0xffffffffu, gy0[k].y, 1), gy0[k].x);
            ta[k] = k == 0 ? gx0[0] : make_float2(__shfl_up_sync(0xffffffffu, gx0[k].y, 1), gx0[k].x);
        }
        const float xc = fmaf(float(i) + 0.5f, F.dl, -F.R);
        face_flux_f<1, float2>(pa, p0, ga, gy0, ta, gx0, bc<float2>(xc), yv, F, fy);
        float2 dfx[3], dfy[3];
        for (int k = 0; k < 3; ++k)
        {
            const float right = __shfl_down_sync(0xffffffffu, fy[k].x, 1);
            dfy[k] = vsub(make_float2(fy[k].y, right), fy[k]);
            dfx[k] = vsub(fxp[k], fxm[k]);
        }
        if constexpr (RING == 2)
        {
            if (interior && writes_state<KIND>(A))
            {
                if (!tma->broken)
                {
                    RawRow2 own;
                    tring_row<KIND>(*tma, i, lane, own);
                    for (int k = 0; k < 3; ++k)
                    {
                        cin.u[k] = own.u[k];
                        cin.d[k] = own.d[k];
                    }
                }
                else load_cell_in<KIND>(A, size_t(i) * N + jg, NN, cin);
            }
        }
        else if constexpr (RING == 1)
        {
            if (interior && writes_state<KIND>(A))
            {
                RawRow2 own;
                ring2_row<KIND>(ring, i, lane, own, slot0);
                for (int k = 0; k < 3; ++k)
                {
                    cin.u[k] = own.u[k];
                    cin.d[k] = own.d[k];
                }
            }
        }
        if (interior)
            mixed_cell2<KIND, DIAG>(A, bc<float2>(xc), yc, p0, dfx, dfy, bf, dtf, size_t(i) * N + jg, NN, cin,
                                    local_max, acc);

        for (int k = 0; k < 3; ++k)
        {
            p0[k] = p1[k];
            p1[k] = p2[k];
            gx0[k] = gx1[k];
            gy0[k] = gy1[k];
            fxm[k] = fxp[k];
            l0[k] = l1[k];
        }
        slot0 = slot0 == RING_ROWS - 1 ? 0 : slot0 + 1;
    }
    // the rows fetched beyond the strip are never read, but no copy may land
    // in shared memory after the warp is gone
    if constexpr (RING == 1) cp_async_wait_all();
    if constexpr (RING == 2) tring_drain(*tma);
    if constexpr (DIAG) diag_flush(A, acc);
    if (A.amax) flush_speed_key(A, local_max.key());
}

// ------------------------------------------------------------- clock
struct ClockArgs
{
    double R, dl, cfl, softening_length, mass_ratio, eccentricity, omega;
    int dt_mode, rk_order;
    int end_step;     // 1: finish the step that just ran (advance time, iteration)
    int begin_step;   // 1: choose dt and stage binaries of the next step
    mara_minidisk_diagnostics* diag;   // optional: integrate the step's rates (end), clear them (begin)
    // mixed CFL mode: the reduction left the fastest cell's speed key in
    // max_wavespeed; at the end of a step it becomes that cell's FP64 wavespeed
    // in the state u_key[key_state] (the step's result)
    int wavespeed_key, key_state;
    const double* u_key[2];
    int N, n, level;
    double rs2, mach;
    int binaries;     // begin_step: 1 = solve both stage binaries here; 0 = the sweeps' binary jobs do
};

// iso2d::fastest_wavespeed at the cell-centre sound speed, FP64, of cell c of
// the SoA state u (the form of the FP64 stage kernels' reduction)
__device__ inline double cell_wavespeed(const double* u, size_t NN, int N, int n, int level, double R, double rs2,
                                        double mach, size_t c)
{
    const int i = int(c / N), j = int(c % N);
    const uint64_t bi = uint64_t(i / n), bj = uint64_t(j / n);
    const int ki = i - int(bi) * n, kj = j - int(bj) * n;
    const double x = 0.5 * (vertex(R, n, level, bi, ki) + vertex(R, n, level, bi, ki + 1));
    const double y = 0.5 * (vertex(R, n, level, bj, kj) + vertex(R, n, level, bj, kj + 1));
    const double cs = sqrt(-(-1.0 / sqrt((x * x + y * y) + rs2)) / mach / mach);
    const double vx = u[NN + c] / u[c], vy = u[2 * NN + c] / u[c];
    return fmax(fmax(fabs(vx - cs), fabs(vx + cs)), fmax(fabs(vy - cs), fabs(vy + cs)));
}

// Complete the rate rows of the step that ran (torques and power from the
// force sums and the binary at each stage time) and add them to the time
// integrals with the RK weights of the update.
__device__ inline void finish_diagnostics(const mara_minidisk_clock* c, const ClockArgs& a)
{
    mara_minidisk_diagnostics* d = a.diag;
    const double t = c->time, dt = c->dt;
    for (int s = 0; s < a.rk_order; ++s)
    {
        double* r = d->rate[s];
        const Binary b = binary_state(a.mass_ratio, a.eccentricity, a.omega, s == 0 ? t : t + dt);
        r[13] = b.x1 * r[7] - b.y1 * r[6];
        r[14] = b.x2 * r[9] - b.y2 * r[8];
        r[15] = (r[6] * b.vx1 + r[7] * b.vy1) + (r[8] * b.vx2 + r[9] * b.vy2);
    }
    for (int k = 0; k < MARA_DIAG_COUNT; ++k)
    {
        if (k == 11 || k == 12)
            d->integral[k] = d->rate[0][k];
        else
            d->integral[k] += a.rk_order == 2 ? dt * (0.5 * (d->rate[0][k] + d->rate[1][k])) : dt * d->rate[0][k];
    }
    d->steps += 1;
}

__device__ inline void store_binary(double* dst, const Binary& b)
{
    dst[0] = b.m1; dst[1] = b.x1; dst[2] = b.y1; dst[3] = b.m2; dst[4] = b.x2; dst[5] = b.y2;
}

// One clock update: finish the step that just ran (RK2 time average,
// iteration count) and/or choose the next dt and the stage binaries.
// The parts of one clock update. `lanes` threads of one warp may share the
// begin-step work: lane 0 does everything else, lane 1 (when present)
// computes the second stage's binary while lane 0 computes the first.
// The time after an RK2 step from t with step dt: the weighted_sum of the
// stage times (one function for the clock and the sweeps' binary job, so
// that both form the same double)
__device__ inline double rk2_end_time(double t, double dt)
{
    const double t2 = (t + dt) + dt;
    return t * 0.5 + t2 * (1.0 - 0.5);
}

__device__ inline void store_binary(double* dst, const Binary& b);

// A sweep launch's binary job (Args::side_binary), by thread 0 (job 0) and
// thread 32 (job 1; thread 1 where the block is a single warp) of block 0: the FP64 Kepler solves that the clock kernel
// would otherwise run between the steps. Stage 1 runs both solves of the
// step on two warps at once, overlapped with its own sweep; stage 2 only
// moves the second into place. Memory written here is read by later
// launches only.
static __device__ __noinline__ void side_binary_job(const Args& A, int job)
{
    mara_minidisk_clock* c = const_cast<mara_minidisk_clock*>(A.clock);
    const double t = c->time, dt = c->dt;
    if (A.side_binary == 1)
    {
        if (job == 0) store_binary(c->binary[1], binary_state(A.mass_ratio, A.eccentricity, A.omega, t + dt));
        else store_binary(A.next_binary, binary_state(A.mass_ratio, A.eccentricity, A.omega, rk2_end_time(t, dt)));
    }
    else if (job == 0)
    {
        for (int k = 0; k < 6; ++k) c->binary[0][k] = A.next_binary[k];
    }
}

__device__ inline void clock_end_step(mara_minidisk_clock* c, const ClockArgs& a)
{
    if (a.diag) finish_diagnostics(c, a);
    if (a.wavespeed_key)
    {
        const unsigned long long key = __double_as_longlong(c->max_wavespeed);
        if (key != 0ull)
        {
            const size_t NN = size_t(a.N) * a.N;
            c->max_wavespeed = cell_wavespeed(a.u_key[a.key_state], NN, a.N, a.n, a.level, a.R, a.rs2, a.mach,
                                              size_t(unsigned(key)));
        }
    }
    double t = c->time, dt = c->dt;
    if (a.rk_order == 2)
    {
        c->time = rk2_end_time(t, dt);   // weighted_sum of the RK2 solution times
    }
    else
    {
        c->time = t + dt;
    }
    c->iteration += 1;
}

__device__ inline double clock_choose_dt(const mara_minidisk_clock* c, const ClockArgs& a)
{
    const double t = c->time;
    if (a.dt_mode == MARA_DT_FORMULA_HELD) return c->dt;   // the batch's dt, chosen by its first step
    if (a.dt_mode == MARA_DT_FORMULA)
    {
        // problems/minidisk.cpp:204-206
        double vmax = sqrt(1.0 * 0.5 / a.softening_length);
        double cfl = a.cfl * fmin(1.0, 0.01 + t / 0.05);
        return a.dl / vmax * cfl;
    }
    return a.cfl * a.dl / c->max_wavespeed;   // scheme_mhd_v1.cpp:287 form
}

// One clock update: finish the step that just ran (RK2 time average,
// iteration count) and/or choose the next dt and the stage binaries.
// Call from `lanes` (1 or 2) consecutive threads of one warp, lane = 0, 1;
// two lanes are an aligned pair (threads 2k and 2k + 1 of a warp).
__device__ inline void advance_clock(mara_minidisk_clock* c, const ClockArgs& a, int lane = 0, int lanes = 1)
{
    const unsigned pair = 0x3u << (threadIdx.x & 30u);
    if (lane == 0)
    {
        if (a.end_step) clock_end_step(c, a);
        if (a.begin_step) c->dt = clock_choose_dt(c, a);
    }
    if (lanes > 1) __syncwarp(pair);
    if (a.begin_step)
    {
        const double t = c->time, dt = c->dt;
        if (a.binaries)
            for (int s = lane; s < 2; s += lanes)
                store_binary(c->binary[s], binary_state(a.mass_ratio, a.eccentricity, a.omega, s == 0 ? t : t + dt));
        if (lanes > 1) __syncwarp(pair);
        if (lane == 0)
        {
            c->max_wavespeed = 0.0;
            if (a.diag)
                for (int k = 0; k < 2 * MARA_DIAG_COUNT; ++k) a.diag->rate[k / MARA_DIAG_COUNT][k % MARA_DIAG_COUNT] = 0.0;
        }
    }
}

// ------------------------------------------------------------- host helpers (minidisk.cu)
int check_params(const mara_minidisk_params* sd);
Args base_args(const mara_minidisk_params* sd);
ClockArgs clock_args(const mara_minidisk_params* sd, int dt_mode, int rk_order, int end_step, int begin_step);
int grid_stage(Args A, int kind, cudaStream_t s);
int clock_init(const mara_minidisk_params* sd, const double* u, double time, mara_minidisk_clock* clock,
               int precision, cudaStream_t s, double* u_copy = nullptr);
int advance_impl(const mara_minidisk_params* sd, double* u, mara_minidisk_clock* clock, int32_t steps,
                 int32_t rk_order, int32_t precision, int32_t dt_mode, void* workspace,
                 mara_minidisk_diagnostics* diag, void* stream, double* final_out);

} // namespace md
} // namespace mara
