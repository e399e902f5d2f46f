// 2D Cartesian special-relativistic hydrodynamics on a uniform square mesh
// (the relativistic shock-tube benchmark). The reference has no such scheme;
// it is composed from the reference's own pieces in the pattern of its
// minidisk scheme: srhd::recover_primitive per cell, generalised-minmod
// slopes of the primitives (scheme_plm_gradient.hpp:44-70), face states
// p -/+ g/2 (minidisk_scheme.cpp:238-240), srhd::riemann_hlle fluxes
// (physics_srhd.hpp:489-497), u -= (dFx + dFy) dt/dl, RK2 by
// control::advance_runge_kutta (app_control.hpp:178-183). Zero-gradient
// boundaries; dt = cfl * dl / max outer wavespeed of the step's initial state.
//
// Per stage:
//   tube_c2p_kernel   conserved -> primitive P[5][N^2] (FP64 Newton; start from
//                     p = 0, the learned guess, or the previous stage's
//                     pressure); fastest wavespeed reduced into the clock
//   tube_flux_kernel  16x32 tile: P with a 2-cell halo in shared memory, slopes,
//                     HLLE on every face of the tile, update (+ RK2 average)
// State: SoA [4][N][N] (D, S1, S2, tau), x slow, y contiguous.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include "common.cuh"
#include "srhd_mlp.cuh"
#include "srhd_physics.cuh"

namespace mara {
namespace tube {

using srhd::SPrim;

struct Clock
{
    double time;
    double dt;
    unsigned long long amax;      // fastest wavespeed (double bits)
    int64_t iteration;
    unsigned long long failures;  // zones whose recovery failed
    unsigned long long newton;    // FP64 Newton iterations summed over all recoveries
    unsigned long long riemann;   // HLLC faces whose contact speed was rejected (HLLE flux used there)
};

enum Guess { GUESS_ZERO = 0, GUESS_MLP = 1, GUESS_PREVIOUS = 2 };

struct C2P
{
    int N;
    double gamma, floor;
    const double* u;
    double* P;                 // [5][N^2]; holds the previous pressure on entry for GUESS_PREVIOUS
    const mlp::Weights* mlp;
    int guess, refine32, budget;
    Clock* clock;
    int reduce_speed;
};

__device__ inline void finish_cell(const C2P& a, int64_t c, const srhd::Zone& z, double guess, double& m,
                                   unsigned long long& bad, unsigned long long& its)
{
    const int64_t NN = int64_t(a.N) * a.N;
    double prim[5] = {0, 0, 0, 0, 0};
    int it = 0, it2 = 0;
    int st;
    if (a.guess == GUESS_ZERO && a.refine32 == 0)
        st = srhd::newton(z, a.gamma, a.floor, 0.0, 50, prim, it);
    else
    {
        if (a.refine32 > 0) guess = srhd::refine_fp32(z, a.gamma, guess, a.refine32);
        st = srhd::newton_fast(z, a.gamma, a.floor, guess, a.budget, prim, it);
        if (st != 0)
        {
            st = srhd::newton(z, a.gamma, a.floor, 0.0, 50, prim, it2);
            it += it2;
        }
    }
    its += it;
    if (st != 0) ++bad;
    for (int k = 0; k < 5; ++k) a.P[k * NN + c] = prim[k];
    if (a.reduce_speed && st == 0)
    {
        SPrim<double> p{prim[0], {prim[1], prim[2], prim[3]}, prim[4]};
        for (int axis = 0; axis < 2; ++axis)
        {
            double am, ap;
            srhd::outer_speeds(p, axis, a.gamma, am, ap);
            m = fmax(m, fmax(fabs(am), fabs(ap)));
        }
    }
}

__device__ inline void reduce_out(const C2P& a, double m, unsigned long long bad, unsigned long long its)
{
    for (int o = 16; o > 0; o >>= 1)
    {
        m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
        bad += __shfl_xor_sync(0xffffffffu, bad, o);
        its += __shfl_xor_sync(0xffffffffu, its, o);
    }
    if ((threadIdx.x & 31) == 0)
    {
        if (a.reduce_speed) atomicMax(&a.clock->amax, (unsigned long long)__double_as_longlong(m));
        if (bad) atomicAdd(&a.clock->failures, bad);
        atomicAdd(&a.clock->newton, its);
    }
}

__global__ void tube_c2p_kernel(const C2P a)
{
    const int64_t NN = int64_t(a.N) * a.N;
    double m = 0.0;
    unsigned long long bad = 0, its = 0;
    for (int64_t c = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; c < NN; c += int64_t(gridDim.x) * blockDim.x)
    {
        srhd::Zone z{a.u[c], a.u[NN + c], a.u[2 * NN + c], 0.0, a.u[3 * NN + c]};
        const double guess = a.guess == GUESS_PREVIOUS ? a.P[4 * NN + c] : 0.0;
        finish_cell(a, c, z, guess, m, bad, its);
    }
    reduce_out(a, m, bad, its);
}

// Learned guess: kZones cells per CTA through the BF16 MLP, then the polish.
__global__ void __launch_bounds__(mlp::kThreads) tube_c2p_mlp_kernel(const C2P a)
{
    __shared__ mlp::Shared sm;
    mlp::begin(*a.mlp, sm);
    uint32_t phase = 0;
    const int64_t NN = int64_t(a.N) * a.N;
    double m = 0.0;
    unsigned long long bad = 0, its = 0;
    for (int64_t base = int64_t(blockIdx.x) * mlp::kZones; base < NN; base += int64_t(gridDim.x) * mlp::kZones)
    {
        __syncthreads();
        for (int t = threadIdx.x; t < mlp::kZones; t += blockDim.x)
        {
            const int64_t c = base + t;
            float f[4] = {0.f, 0.f, 0.f, 0.f};
            if (c < NN) mlp::features(a.u[c], a.u[NN + c], a.u[2 * NN + c], 0.0, a.u[3 * NN + c], f);
            mlp::stage_features(sm, t, f);
        }
        __syncthreads();
        mlp::forward(sm, phase);
        __syncthreads();
        for (int t = threadIdx.x; t < mlp::kZones; t += blockDim.x)
        {
            const int64_t c = base + t;
            if (c >= NN) continue;
            srhd::Zone z{a.u[c], a.u[NN + c], a.u[2 * NN + c], 0.0, a.u[3 * NN + c]};
            finish_cell(a, c, z, mlp::pressure_from_output(sm.out[t], z.D, z.S1, z.S2, z.S3, z.tau), m, bad, its);
        }
    }
    mlp::end(sm);
    reduce_out(a, m, bad, its);
}

__global__ void dt_kernel(Clock* c, double cfl, double dl, int begin)
{
    if (threadIdx.x != 0) return;
    if (begin) { c->amax = 0ull; return; }
    c->dt = cfl * dl / __longlong_as_double((long long)c->amax);
}

__global__ void clock_end_kernel(Clock* c)
{
    if (threadIdx.x != 0) return;
    const double t = c->time, dt = c->dt;
    const double t2 = (t + dt) + dt;
    c->time = t * 0.5 + t2 * (1 - 0.5);
    c->iteration += 1;
}

// ------------------------------------------------------------- flux + update
constexpr int TX = 16, TY = 32, NT = 256;
constexpr int EX = TX + 4, EY = TY + 4;

struct Flux
{
    int N;
    double gamma, theta, dl;
    const double* P;
    const double* u_in;
    const double* u_avg;
    double* u_out;
    Clock* clock;
    int tiles_y;
};

template<typename R>
struct TileSmem
{
    R p[5][EX][EY];
    R fx[4][TX + 1][TY];
    R fy[4][TX][TY + 1];
};

__device__ inline double plm(double yl, double y0, double yr, double theta)
{
    double a = (y0 - yl) * theta, b = (yr - yl) * 0.5, c = (yr - y0) * theta;
    double m = fmin(fmin(fabs(a), fabs(b)), fabs(c));
    long long sa = __double_as_longlong(a), sb = __double_as_longlong(b), sc = __double_as_longlong(c);
    return ((sa ^ sb) | (sa ^ sc)) < 0 ? 0.0 : copysign(m, a);
}

__device__ inline float plm(float yl, float y0, float yr, float theta)
{
    float a = (y0 - yl) * theta, b = (yr - yl) * 0.5f, c = (yr - y0) * theta;
    float m = fminf(fminf(fabsf(a), fabsf(b)), fabsf(c));
    int sa = __float_as_int(a), sb = __float_as_int(b), sc = __float_as_int(c);
    return ((sa ^ sb) | (sa ^ sc)) < 0 ? 0.0f : copysignf(m, a);
}

// SOLVER: 0 HLLE, 1 HLLC (riemann_solver, physics_srhd.hpp:377-487)
template<typename R, int SOLVER>
__global__ void __launch_bounds__(NT) tube_flux_kernel(const Flux A)
{
    extern __shared__ __align__(16) unsigned char raw[];
    TileSmem<R>& S = *reinterpret_cast<TileSmem<R>*>(raw);
    const int tid = threadIdx.x;
    const int N = A.N;
    const int64_t NN = int64_t(N) * N;
    const int gx0 = (blockIdx.x / A.tiles_y) * TX, gy0 = (blockIdx.x % A.tiles_y) * TY;
    const R theta = R(A.theta), gm = R(A.gamma);

    for (int e = tid; e < EX * EY; e += NT)
    {
        const int ei = e / EY, ej = e - (e / EY) * EY;
        const int i = min(max(gx0 + ei - 2, 0), N - 1), j = min(max(gy0 + ej - 2, 0), N - 1);   // zero gradient
        const int64_t c = int64_t(i) * N + j;
        for (int k = 0; k < 5; ++k) S.p[k][ei][ej] = R(A.P[k * NN + c]);
    }
    __syncthreads();

    // faces: x face (fi, j) between tile cells (fi-1, j) and (fi, j) -> halo (fi+1, j+2), (fi+2, j+2)
    unsigned rejected = 0;
    for (int e = tid; e < (TX + 1) * TY + TX * (TY + 1); e += NT)
    {
        const bool xf = e < (TX + 1) * TY;
        int a0, a1, b0, b1;
        if (xf)
        {
            const int fi = e / TY, j = e - (e / TY) * TY;
            a0 = fi + 1; a1 = j + 2; b0 = fi + 2; b1 = j + 2;
        }
        else
        {
            const int q = e - (TX + 1) * TY;
            const int i = q / (TY + 1), fj = q - (q / (TY + 1)) * (TY + 1);
            a0 = i + 2; a1 = fj + 1; b0 = i + 2; b1 = fj + 2;
        }
        const int d0 = xf ? 1 : 0, d1 = xf ? 0 : 1;
        SPrim<R> L, Rr;
        R l[5], r[5];
        for (int k = 0; k < 5; ++k)
        {
            const R pa = S.p[k][a0][a1], pb = S.p[k][b0][b1];
            const R ga = plm(S.p[k][a0 - d0][a1 - d1], pa, pb, theta);
            const R gb = plm(pa, pb, S.p[k][b0 + d0][b1 + d1], theta);
            l[k] = pa + R(0.5) * ga;
            r[k] = pb - R(0.5) * gb;
        }
        L = SPrim<R>{l[0], {l[1], l[2], l[3]}, l[4]};
        Rr = SPrim<R>{r[0], {r[1], r[2], r[3]}, r[4]};
        R F[5];
        if (SOLVER == 1) rejected += srhd::hllc(L, Rr, xf ? 0 : 1, gm, F);
        else srhd::hlle(L, Rr, xf ? 0 : 1, gm, F);
        const int comp[4] = {0, 1, 2, 4};
        if (xf)
        {
            const int fi = e / TY, j = e - (e / TY) * TY;
            for (int q = 0; q < 4; ++q) S.fx[q][fi][j] = F[comp[q]];
        }
        else
        {
            const int q0 = e - (TX + 1) * TY;
            const int i = q0 / (TY + 1), fj = q0 - (q0 / (TY + 1)) * (TY + 1);
            for (int q = 0; q < 4; ++q) S.fy[q][i][fj] = F[comp[q]];
        }
    }
    if (SOLVER == 1)
    {
        for (int o = 16; o > 0; o >>= 1) rejected += __shfl_xor_sync(0xffffffffu, rejected, o);
        if ((tid & 31) == 0 && rejected) atomicAdd(&A.clock->riemann, (unsigned long long)rejected);
    }
    __syncthreads();

    const double dt = A.clock->dt;
    const float dt_over_dl = float(dt / A.dl);
    for (int e = tid; e < TX * TY; e += NT)
    {
        const int i = e / TY, j = e - (e / TY) * TY;
        const int gi = gx0 + i, gj = gy0 + j;
        if (gi >= N || gj >= N) continue;
        const int64_t c = int64_t(gi) * N + gj;
        for (int q = 0; q < 4; ++q)
        {
            double v;
            if (sizeof(R) == sizeof(double))
            {
                const double dfx = double(S.fx[q][i + 1][j]) - double(S.fx[q][i][j]);
                const double dfy = double(S.fy[q][i][j + 1]) - double(S.fy[q][i][j]);
                v = A.u_in[q * NN + c] - (dfx + dfy) * dt / A.dl;
            }
            else
            {
                const float d = (float(S.fx[q][i + 1][j]) - float(S.fx[q][i][j])) + (float(S.fy[q][i][j + 1]) - float(S.fy[q][i][j]));
                v = A.u_in[q * NN + c] - double(d * dt_over_dl);
            }
            if (A.u_avg) v = A.u_avg[q * NN + c] * 0.5 + v * (1 - 0.5);
            A.u_out[q * NN + c] = v;
        }
    }
}

template<typename R, int SOLVER>
int launch_flux(const Flux& F, cudaStream_t s)
{
    static PerDeviceOnce once;
    int dev = 0;
    MARA_CUDA(cudaGetDevice(&dev));
    if (int r = once.run(dev, []() -> int {
            MARA_CUDA(cudaFuncSetAttribute(tube_flux_kernel<R, SOLVER>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           int(sizeof(TileSmem<R>))));
            return MARA_OK;
        }))
        return r;
    Flux A = F;
    A.tiles_y = (A.N + TY - 1) / TY;
    const int tiles = ((A.N + TX - 1) / TX) * A.tiles_y;
    tube_flux_kernel<R, SOLVER><<<tiles, NT, sizeof(TileSmem<R>), s>>>(A);
    return launch_status("tube_flux_kernel");
}

int launch_flux(const Flux& F, int precision, int solver, cudaStream_t s)
{
    if (precision == MARA_MIXED) return solver ? launch_flux<float, 1>(F, s) : launch_flux<float, 0>(F, s);
    return solver ? launch_flux<double, 1>(F, s) : launch_flux<double, 0>(F, s);
}

inline int blocks_for(int64_t n) { return int(std::min<int64_t>((n + 255) / 256, 152 * 16)); }

} // namespace tube
} // namespace mara

using namespace mara;
using namespace mara::tube;

extern "C" {

int64_t mara_srhd_tube_clock_bytes(void) { return int64_t(sizeof(Clock)); }

int64_t mara_srhd_tube_workspace_bytes(int32_t N)
{
    if (N < 4 || N > 16384) return -1;
    const int64_t NN = int64_t(N) * N;
    return 5 * NN * 8 + 4 * NN * 8 + 256;     // primitives + the stage-1 state
}

int mara_srhd_tube_initial(int32_t N, double angle, double rho_l, double p_l, double rho_r, double p_r,
                           double gamma_law_index, double* u, void* clock, void* stream)
{
    MARA_REQUIRE(N >= 4 && u && clock, "mara_srhd_tube_initial: bad argument");
    // computed on the host (one-time set-up) and copied in
    const int64_t NN = int64_t(N) * N;
    double* h = new double[4 * NN];
    const double c = std::cos(angle), s = std::sin(angle);
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j)
        {
            const double x = (i + 0.5) / N, y = (j + 0.5) / N;
            const bool left = (x - 0.5) * c + (y - 0.5) * s < 0.0;
            const double rho = left ? rho_l : rho_r, p = left ? p_l : p_r;
            const double W = std::sqrt(1.0 + 0.0);
            const double D = rho * W;
            const double hh = (rho * 1.0 + p * (1.0 + 1.0 / (gamma_law_index - 1.0))) / rho;
            const int64_t k = int64_t(i) * N + j;
            h[k] = D;
            h[NN + k] = D * hh * 0.0 / 1.0;
            h[2 * NN + k] = D * hh * 0.0 / 1.0;
            h[3 * NN + k] = D * (hh * W - 1.0 * 1.0) - p;
        }
    cudaStream_t st = as_stream(stream);
    cudaError_t e = cudaMemcpyAsync(u, h, sizeof(double) * 4 * NN, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    delete[] h;
    if (e != cudaSuccess) return cuda_fail(e, "mara_srhd_tube_initial copy");
    Clock cl;
    std::memset(&cl, 0, sizeof cl);
    MARA_CUDA(cudaMemcpyAsync(clock, &cl, sizeof cl, cudaMemcpyHostToDevice, st));
    MARA_CUDA(cudaStreamSynchronize(st));
    return MARA_OK;
}

int mara_srhd_tube_advance(int32_t N, double* u, void* clock, int32_t steps, double cfl, double plm_theta,
                           double gamma_law_index, double temperature_floor, int32_t precision, int32_t guess,
                           const void* mlp_weights, int32_t refine32, int32_t riemann_solver, void* workspace,
                           void* stream)
{
    MARA_REQUIRE(N >= 4 && u && clock && workspace, "mara_srhd_tube_advance: bad argument");
    MARA_REQUIRE(riemann_solver == 0 || riemann_solver == 1, "mara_srhd_tube_advance: riemann_solver must be 0 or 1");
    MARA_REQUIRE(precision == MARA_FP64 || precision == MARA_MIXED, "mara_srhd_tube_advance: bad precision");
    MARA_REQUIRE(guess >= GUESS_ZERO && guess <= GUESS_PREVIOUS, "mara_srhd_tube_advance: bad guess kind");
    MARA_REQUIRE(guess != GUESS_MLP || mlp_weights, "mara_srhd_tube_advance: the learned guess needs weights");
    MARA_REQUIRE(refine32 >= 0 && refine32 <= 16, "mara_srhd_tube_advance: refine32 must be in [0, 16]");
    cudaStream_t s = as_stream(stream);
    Clock* c = static_cast<Clock*>(clock);
    const int64_t NN = int64_t(N) * N;
    double* P = static_cast<double*>(workspace);
    double* u1 = P + 5 * NN;
    const double dl = 1.0 / double(N);

    C2P a;
    a.N = N;
    a.gamma = gamma_law_index;
    a.floor = temperature_floor;
    a.P = P;
    a.mlp = static_cast<const mlp::Weights*>(mlp_weights);
    a.guess = guess;
    a.refine32 = refine32;
    a.budget = 12;
    a.clock = c;
    Flux f;
    std::memset(&f, 0, sizeof f);
    f.N = N;
    f.gamma = gamma_law_index;
    f.theta = plm_theta;
    f.dl = dl;
    f.P = P;
    f.clock = c;
    auto c2p = [&] (const double* state, int reduce) {
        a.u = state;
        a.reduce_speed = reduce;
        if (guess == GUESS_MLP)
        {
            const int blocks = int(std::min<int64_t>((NN + mlp::kZones - 1) / mlp::kZones, 152 * 8));
            tube_c2p_mlp_kernel<<<blocks, mlp::kThreads, 0, s>>>(a);
        }
        else
            tube_c2p_kernel<<<blocks_for(NN), 256, 0, s>>>(a);
        return launch_status("tube c2p kernel");
    };
    // the warm start needs a pressure in P: start it from p = 0 on each call
    if (guess == GUESS_PREVIOUS) MARA_CUDA(cudaMemsetAsync(P + 4 * NN, 0, NN * sizeof(double), s));
    for (int step = 0; step < steps; ++step)
    {
        dt_kernel<<<1, 32, 0, s>>>(c, cfl, dl, 1);
        if (int r = c2p(u, 1)) return r;
        dt_kernel<<<1, 32, 0, s>>>(c, cfl, dl, 0);
        if (int r = launch_status("tube dt_kernel")) return r;
        f.u_in = u; f.u_avg = nullptr; f.u_out = u1;
        if (int r = launch_flux(f, precision, riemann_solver, s)) return r;
        if (int r = c2p(u1, 0)) return r;
        f.u_in = u1; f.u_avg = u; f.u_out = u;
        if (int r = launch_flux(f, precision, riemann_solver, s)) return r;
        clock_end_kernel<<<1, 32, 0, s>>>(c);
        if (int r = launch_status("tube clock_end_kernel")) return r;
    }
    return MARA_OK;
}

} // extern "C"
