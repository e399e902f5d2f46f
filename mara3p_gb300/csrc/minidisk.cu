// Locally-isothermal binary-minidisk Godunov update on the GPU.
//
// One CTA updates a TX x TY tile of the mesh (x rows slow, y contiguous):
//   phase 1  load the (TX+4) x (TY+4) halo tile of the stage state (periodic
//            wrap), recover primitives into shared memory
//   phase 2  PLM limited slopes along x and y (scheme_plm_gradient.hpp:44-70)
//   phase 3  HLLE + viscous fluxes on the TX+1 x-face rows and TY+1 y-face
//            columns (problems/minidisk_scheme.cpp:222-288, physics_iso2d.hpp:156-173)
//   phase 4  flux divergence + gravity, sink, rotating-frame and buffer
//            sources, stage update (problems/minidisk_scheme.cpp:294-355),
//            optionally fused with the RK2 average and the CFL wavespeed
//            reduction of the new state.
//
// Two arithmetic paths share the template:
//   FP64   (R = double): the drop-in path. Every expression keeps the
//          reference's evaluation order; only FMA contraction and CUDA's libm
//          (sqrt/exp/tanh, x^1.5 as x*sqrt(x), x^3 as x*x*x) differ.
//   MIXED  (R = float): reconstruction, fluxes and sources in FP32; the state
//          stays FP64 in HBM and is accumulated in FP64. RK2 keeps only the
//          FP32 stage-1 increment d1 = dt*L(u0) between stages; stage 2 uses
//          u1 = f32(u0) + d1 for its fluxes and writes u0 + (d1 + d2)/2 in FP64.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <cstdint>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <atomic>
#include <mutex>
#include <string>
#include "minidisk_device.cuh"

namespace mara {
namespace md {

// Workspace tail of mixed RK2: the next step's stage-1 binary (6 doubles),
// padded to 64 bytes.
constexpr int64_t kNextBinaryBytes = 64;

// ------------------------------------------------------------- shared layout
template<typename R>
struct Smem
{
    // primitives of the halo tile; in the FP64 path an interior tile's raw
    // state lands here first, by one TMA copy (box 36 x 20 x 3 of [3][N][N])
    __align__(128) R p[3][EX][EY];
    R gx[3][GX][GY];       // x slopes of halo-tile cells [1, TX+3) x [1, TY+3)
    R gy[3][GX][GY];       // y slopes, same cells
    R fx[3][TX + 1][TY];   // x-face fluxes
    R fy[3][TX][TY + 1];   // y-face fluxes
    R xv[TX + 1], xc[TX], yv[TY + 1], yc[TY];
    double wmax[NT / 32];
    unsigned long long tma_bar;   // completion barrier of the tile copy
};

// Bounded wait on the tile copy's barrier (phase 0): false if it timed out.
__device__ inline bool tile_copy_wait(unsigned long long* bar)
{
    const uint32_t addr = uint32_t(__cvta_generic_to_shared(bar));
    uint32_t done = 0;
    for (int it = 0; it < (1 << 22) && !done; ++it)
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}" : "=r"(done) : "r"(addr), "r"(0));
    return done != 0;
}

template<typename R>
__device__ inline R to_r(double v) { return R(v); }

// ------------------------------------------------------------- stage kernel
// tmap: the state [3][N][N] as a 3D tensor (columns, rows, components) with a
// 36 x 20 x 3 box, used by FP64 tiles that need no periodic wrap (A.use_tma).
template<typename R, int KIND>
__global__ void __launch_bounds__(NT) stage_kernel(const Args A, const __grid_constant__ CUtensorMap tmap)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Smem<R>& S = *reinterpret_cast<Smem<R>*>(smem_raw);
    const int tid = threadIdx.x;
    const int tx = blockIdx.x / A.tiles_y, ty = blockIdx.x % A.tiles_y;
    const int gx0 = tx * TX, gy0 = ty * TY;
    const int N = A.N;
    const size_t NN = size_t(N) * N;

    // FP64 interior tile: one bulk tensor copy of the raw halo tile into S.p,
    // issued first so that it runs while the coordinates are computed. The
    // box's first coordinate (gy0 - 2 doubles) is a multiple of 16 bytes.
    bool tma = false;
    if constexpr (KIND == K_FP64)
    {
        tma = A.use_tma && gx0 >= 2 && gx0 + TX + 2 <= N && gy0 >= 2 && gy0 + TY + 2 <= N &&
              (__cvta_generic_to_shared(&S.p[0][0][0]) & 127) == 0;
        if (tma)
        {
            const uint32_t bar = uint32_t(__cvta_generic_to_shared(&S.tma_bar));
            if (tid == 0)
            {
                asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(bar), "r"(1));
                asm volatile("fence.mbarrier_init.release.cluster;");
            }
            __syncthreads();
            if (tid == 0)
            {
                const uint32_t dst = uint32_t(__cvta_generic_to_shared(&S.p[0][0][0]));
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                             :: "r"(bar), "r"(uint32_t(sizeof(S.p))));
                asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
                             " [%0], [%1, {%2, %3, %4}], [%5];"
                             :: "r"(dst), "l"(reinterpret_cast<uint64_t>(&tmap)), "r"(gy0 - 2), "r"(gx0 - 2), "r"(0),
                                "r"(bar)
                             : "memory");
            }
        }
    }

    // coordinates of this tile's vertices and centres: the reference's
    // per-block linspace in FP64 for the FP64 path, x = -R + i*dl in FP32 for
    // the mixed path
    if (sizeof(R) == sizeof(float))
    {
        for (int e = tid; e < (TX + 1) + TX + (TY + 1) + TY; e += NT)
        {
            if (e < TX + 1) S.xv[e] = R(fmaf(float(gx0 + e), A.f.dl, -A.f.R));
            else if (e < 2 * TX + 1) S.xc[e - (TX + 1)] = R(fmaf(float(gx0 + e - (TX + 1)) + 0.5f, A.f.dl, -A.f.R));
            else if (e < 2 * TX + TY + 2) S.yv[e - (2 * TX + 1)] = R(fmaf(float(gy0 + e - (2 * TX + 1)), A.f.dl, -A.f.R));
            else S.yc[e - (2 * TX + TY + 2)] = R(fmaf(float(gy0 + e - (2 * TX + TY + 2)) + 0.5f, A.f.dl, -A.f.R));
        }
    }
    else
    for (int e = tid; e < (TX + 1) + TX + (TY + 1) + TY; e += NT)
    {
        int q = e;
        if (q < TX + 1 + TX)
        {
            bool is_center = q > TX;
            int k = is_center ? q - (TX + 1) : q;
            int I = gx0 + k;
            uint64_t b; int kk;
            if (KIND == K_BLOCK) { b = A.bi; kk = I; }
            else { b = uint64_t(min(I / A.n, (1 << A.level) - 1)); kk = I - int(b) * A.n; }
            double v = is_center ? 0.5 * (vertex(A.R, A.n, A.level, b, kk) + vertex(A.R, A.n, A.level, b, kk + 1))
                                 : vertex(A.R, A.n, A.level, b, kk);
            if (is_center) S.xc[k] = to_r<R>(v); else S.xv[k] = to_r<R>(v);
        }
        else
        {
            q -= TX + 1 + TX;
            bool is_center = q > TY;
            int k = is_center ? q - (TY + 1) : q;
            int J = gy0 + k;
            uint64_t b; int kk;
            if (KIND == K_BLOCK) { b = A.bj; kk = J; }
            else { b = uint64_t(min(J / A.n, (1 << A.level) - 1)); kk = J - int(b) * A.n; }
            double v = is_center ? 0.5 * (vertex(A.R, A.n, A.level, b, kk) + vertex(A.R, A.n, A.level, b, kk + 1))
                                 : vertex(A.R, A.n, A.level, b, kk);
            if (is_center) S.yc[k] = to_r<R>(v); else S.yv[k] = to_r<R>(v);
        }
    }

    // phase 1: halo tile -> primitives (in place after the tile copy)
    if (tma && tile_copy_wait(&S.tma_bar))
    {
        for (int e = tid; e < EX * EY; e += NT)
        {
            const int ei = e / EY, ej = e - (e / EY) * EY;
            const double s = S.p[0][ei][ej], m1 = S.p[1][ei][ej], m2 = S.p[2][ei][ej];
            S.p[1][ei][ej] = R(m1 / s);
            S.p[2][ei][ej] = R(m2 / s);
        }
    }
    else
    for (int e = tid; e < EX * EY; e += NT)
    {
        int ei = e / EY, ej = e - (e / EY) * EY;
        R p0, p1, p2;
        if (KIND == K_BLOCK)
        {
            int i = min(gx0 + ei, A.n + 3), j = min(gy0 + ej, A.n + 3);
            const double* q = A.pe + (size_t(i) * (A.n + 4) + j) * 3;
            p0 = R(q[0]); p1 = R(q[1]); p2 = R(q[2]);
        }
        else
        {
            size_t idx = size_t(wrap(gx0 + ei - 2, N)) * N + wrap(gy0 + ej - 2, N);
            double s = __ldg(A.u_in + idx), m1 = __ldg(A.u_in + NN + idx), m2 = __ldg(A.u_in + 2 * NN + idx);
            if (KIND == K_FP64)
            {
                p0 = R(s); p1 = R(m1 / s); p2 = R(m2 / s);
            }
            else
            {
                float fs = d2f(s), f1 = d2f(m1), f2 = d2f(m2);
                if (KIND == K_MIX2)
                {
                    fs += __ldg(A.d1 + idx); f1 += __ldg(A.d1 + NN + idx); f2 += __ldg(A.d1 + 2 * NN + idx);
                }
                float inv = rcp_fast(fs);
                p0 = R(fs); p1 = R(div_corrected(f1, fs, inv)); p2 = R(div_corrected(f2, fs, inv));
            }
        }
        S.p[0][ei][ej] = p0; S.p[1][ei][ej] = p1; S.p[2][ei][ej] = p2;
    }
    __syncthreads();

    // phase 2: slopes
    for (int e = tid; e < GX * GY; e += NT)
    {
        int gi = e / GY, gj = e - (e / GY) * GY;
        for (int k = 0; k < 3; ++k)
        {
            S.gx[k][gi][gj] = cell_slope<R>(S.p[k][gi][gj + 1], S.p[k][gi + 1][gj + 1], S.p[k][gi + 2][gj + 1], A);
            S.gy[k][gi][gj] = cell_slope<R>(S.p[k][gi + 1][gj], S.p[k][gi + 1][gj + 1], S.p[k][gi + 1][gj + 2], A);
        }
    }
    __syncthreads();

    // phase 3: face fluxes
    for (int e = tid; e < NFX + NFY; e += NT)
    {
        R pa[3], pb[3], ga[3], gb[3], ta[3], tb[3], F[3];
        if (e < NFX)
        {
            int fi = e / TY, j = e - (e / TY) * TY;
            // left cell ext (fi+1, j+2) = slope (fi, j+1); right ext (fi+2, j+2) = slope (fi+1, j+1)
            for (int k = 0; k < 3; ++k)
            {
                pa[k] = S.p[k][fi + 1][j + 2]; pb[k] = S.p[k][fi + 2][j + 2];
                ga[k] = S.gx[k][fi][j + 1];    gb[k] = S.gx[k][fi + 1][j + 1];
                ta[k] = S.gy[k][fi][j + 1];    tb[k] = S.gy[k][fi + 1][j + 1];
            }
            face_flux<0>(pa, pb, ga, gb, ta, tb, S.xv[fi], S.yc[j], A, F);
            for (int k = 0; k < 3; ++k) S.fx[k][fi][j] = F[k];
        }
        else
        {
            int q = e - NFX;
            int i = q / (TY + 1), fj = q - (q / (TY + 1)) * (TY + 1);
            // left cell ext (i+2, fj+1) = slope (i+1, fj); right ext (i+2, fj+2) = slope (i+1, fj+1)
            for (int k = 0; k < 3; ++k)
            {
                pa[k] = S.p[k][i + 2][fj + 1]; pb[k] = S.p[k][i + 2][fj + 2];
                ga[k] = S.gy[k][i + 1][fj];    gb[k] = S.gy[k][i + 1][fj + 1];
                ta[k] = S.gx[k][i + 1][fj];    tb[k] = S.gx[k][i + 1][fj + 1];
            }
            face_flux<1>(pa, pb, ga, gb, ta, tb, S.xc[i], S.yv[fj], A, F);
            for (int k = 0; k < 3; ++k) S.fy[k][i][fj] = F[k];
        }
    }
    __syncthreads();

    // phase 4: divergence, sources, update
    double dt;
    double b6[6];
    if (A.clock)
    {
        dt = A.clock->dt;
        for (int k = 0; k < 6; ++k) b6[k] = A.clock->binary[A.stage][k];
    }
    else
    {
        dt = A.dt;
        for (int k = 0; k < 6; ++k) b6[k] = A.bin[k];
    }
    double local_max = 0.0;
    KeyMax local_key;                      // mixed kinds
    float bf[6];
    for (int k = 0; k < 6; ++k) bf[k] = d2f(b6[k]);
    const float dtf = d2f(dt);
    const int cells_x = KIND == K_BLOCK ? A.n : N;

    for (int e = tid; e < TX * TY; e += NT)
    {
        int i = e / TY, j = e - (e / TY) * TY;
        int gi = gx0 + i, gj = gy0 + j;
        if (gi >= cells_x || gj >= cells_x) continue;
        R pc[3] = {S.p[0][i + 2][j + 2], S.p[1][i + 2][j + 2], S.p[2][i + 2][j + 2]};
        R dfx[3], dfy[3];
        for (int k = 0; k < 3; ++k)
        {
            dfx[k] = S.fx[k][i + 1][j] - S.fx[k][i][j];
            dfy[k] = S.fy[k][i][j + 1] - S.fy[k][i][j];
        }

        if (KIND == K_FP64 || KIND == K_BLOCK)
        {
            const double x = S.xc[i], y = S.yc[j];
            double uc[3];
            size_t idx = size_t(gi) * N + gj;
            if (KIND == K_BLOCK)
                for (int k = 0; k < 3; ++k) uc[k] = A.u_in[(size_t(gi) * A.n + gj) * 3 + k];
            else
                for (int k = 0; k < 3; ++k) uc[k] = A.u_in[k * NN + idx];

            // two_body::gravitational_acceleration (physics_two_body.hpp:209-218)
            double dx1 = x - b6[1], dy1 = y - b6[2];
            double t1 = (dx1 * dx1 + dy1 * dy1) + A.rs2;
            double g1 = -1.0 * b6[0] / (t1 * sqrt(t1));
            double dx2 = x - b6[4], dy2 = y - b6[5];
            double t2 = (dx2 * dx2 + dy2 * dy2) + A.rs2;
            double g2 = -1.0 * b6[3] / (t2 * sqrt(t2));
            double ag1x = g1 * dx1, ag1y = g1 * dy1, ag2x = g2 * dx2, ag2y = g2 * dy2;
            // sink_rate_field (problems/minidisk_scheme.cpp:57-65)
            double d1 = 0.0 + dx1 * dx1 + dy1 * dy1;
            double d2 = 0.0 + dx2 * dx2 + dy2 * dy2;
            double sr1 = A.sink_rate * exp(-(d1 * d1 * d1) / A.s6);
            double sr2 = A.sink_rate * exp(-(d2 * d2 * d2) / A.s6);
            // buffer_rate_field (problems/minidisk_scheme.cpp:47-55)
            double rr = sqrt(0.0 + x * x + y * y);
            double br = 0.5 * A.buffer_rate * (1.0 + tanh((rr - A.R) / A.buffer_scale));
            // initial_primitive -> conserved (problems/minidisk_scheme.cpp:87-99)
            double ph = -1.0 / sqrt((x * x + y * y) + A.rs2);
            double r0 = sqrt(x * x + y * y);
            double vp = sqrt(-ph) - A.omega * r0;
            double ui[3] = {1.0, 1.0 * (vp * (-y / r0)), 1.0 * (vp * (x / r0))};
            // coriolis_term / centrifugal_term (problems/minidisk_scheme.cpp:67-76)
            double sig = pc[0];
            double corx = 2.0 * A.omega * double(pc[2]);
            double cory = 2.0 * A.omega * -double(pc[1]);
            double cenx = A.omega * A.omega * x;
            double ceny = A.omega * A.omega * y;
            double sg1[3] = {0.0, sig * ag1x, sig * ag1y};
            double sg2[3] = {0.0, sig * ag2x, sig * ag2y};
            double sf1[3] = {0.0, sig * cenx, sig * ceny};
            double sf2[3] = {0.0, sig * corx, sig * cory};
            double out[3];
            for (int k = 0; k < 3; ++k)
            {
                double ss1 = -uc[k] * sr1;
                double ss2 = -uc[k] * sr2;
                double sb = -(uc[k] - ui[k]) * br;
                double u1 = uc[k] - (double(dfx[k]) + double(dfy[k])) * dt / A.dl
                          + (sg1[k] + sg2[k] + ss1 + ss2 + sf1[k] + sf2[k] + sb) * dt;
                out[k] = u1;
            }
            if (KIND == K_BLOCK)
            {
                for (int k = 0; k < 3; ++k) A.u_out[(size_t(gi) * A.n + gj) * 3 + k] = out[k];
            }
            else
            {
                if (A.u_avg)
                    for (int k = 0; k < 3; ++k) out[k] = A.u_avg[k * NN + idx] * 0.5 + out[k] * (1.0 - 0.5);
                for (int k = 0; k < 3; ++k) A.u_out[k * NN + idx] = out[k];
                if (A.amax)
                {
                    // iso2d::fastest_wavespeed at the cell-centre sound speed
                    double cs = sqrt(-(-1.0 / sqrt((x * x + y * y) + A.rs2)) / A.mach / A.mach);
                    double vx = out[1] / out[0], vy = out[2] / out[0];
                    double a = fmax(fmax(fabs(vx - cs), fabs(vx + cs)), fmax(fabs(vy - cs), fabs(vy + cs)));
                    local_max = fmax(local_max, a);
                }
            }
        }
        else
        {
            size_t idx = size_t(gi) * N + gj;
            const float p3[3] = {float(pc[0]), float(pc[1]), float(pc[2])};
            const float fx3[3] = {float(dfx[0]), float(dfx[1]), float(dfx[2])};
            const float fy3[3] = {float(dfy[0]), float(dfy[1]), float(dfy[2])};
            CellIn<float> cin;
            load_cell_in<KIND>(A, idx, NN, cin);
            mixed_cell<KIND>(A, float(S.xc[i]), float(S.yc[j]), p3, fx3, fy3, bf, dtf, idx, NN, cin, local_key);
        }
    }

    if (A.amax && sizeof(R) == sizeof(float))
    {
        flush_speed_key(A, local_key.key());
    }
    else if (A.amax)
    {
        for (int o = 16; o > 0; o >>= 1) local_max = fmax(local_max, __shfl_xor_sync(0xffffffffu, local_max, o));
        if ((tid & 31) == 0) S.wmax[tid >> 5] = local_max;
        __syncthreads();
        if (tid == 0)
        {
            double m = 0.0;
            for (int w = 0; w < NT / 32; ++w) m = fmax(m, S.wmax[w]);
            atomicMax(A.amax, (unsigned long long)__double_as_longlong(m));
        }
    }
}

// ------------------------------------------------------------- warp-strip sweep (mixed path)
// TMA (two-column form only): rows staged by bulk tensor copies of the stage
// input [3][N][N] (umap, FP64) and, in stage 2, of the FP32 increment (dmap),
// one-row boxes; strips that the boxes cannot reach without wrapping use the
// per-lane ring. The default instantiation (TMA false) has only the per-lane
// ring: measured at 4096^2 it is the faster of the two (0.469 against 0.526
// ms per RK2 step), so bulk copies are an option (mara_minidisk_sweep_tma).
template<int KIND, int COLS, bool DIAG, bool TMA>
__global__ void __launch_bounds__(SW_WARPS * 32) sweep_kernel(const Args A, const __grid_constant__ CUtensorMap umap,
                                                              const __grid_constant__ CUtensorMap dmap)
{
    extern __shared__ __align__(128) unsigned char ring_smem[];  // two-column form: one ring per warp
    int block = int(blockIdx.x);
    if (A.side_binary)
    {
        // block 0 is scheduled first: its binary job overlaps the whole stage
        if (block == 0)
        {
            // job 1 on a second warp, or on lane 1 of a one-warp block
            if (threadIdx.x == 0) side_binary_job(A, 0);
            else if (threadIdx.x == (blockDim.x >= 64 ? 32u : 1u)) side_binary_job(A, 1);
            return;
        }
        block -= 1;
    }
    const int warp = block * int(blockDim.x >> 5) + (threadIdx.x >> 5);
    const int sx = warp / A.tiles_y, sy = warp - sx * A.tiles_y;
    const int i0 = sx * A.sweep_rows;
    if (i0 >= A.N) return;                    // uniform per warp
    if constexpr (COLS == 2)
    {
        unsigned char* base = ring_smem + (threadIdx.x >> 5) * (TMA ? TRING_WARP_BYTES : RING_WARP_BYTES);
        const int i1 = min(i0 + A.sweep_rows, A.N);
        if constexpr (TMA)
        {
            if (tma_strip(sy, A.N) && (smem_u32(base) & 127u) == 0)
            {
                RingT T{base, &umap, &dmap, sy * SW2_COLS - 2, sy * SW2_COLS - 4, 0, 0, 0, false};
                sweep_strip2<KIND, DIAG, 2>(A, i0, i1, sy, Ring2{}, &T);
                return;
            }
        }
        const Ring2 ring{reinterpret_cast<double2*>(base), reinterpret_cast<float2*>(base + RING_U_BYTES)};
        sweep_strip2<KIND, DIAG, 1>(A, i0, i1, sy, ring);
    }
    else sweep_strip<KIND, DIAG>(A, i0, min(i0 + A.sweep_rows, A.N), sy);
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder();

// [3][N][N] field (FP64 or FP32) as a tensor map with a one-row box of
// `cols` columns and all three components (the sweeps' TMA ring)
bool row_tensor_map(const void* base, int N, bool fp64, int cols, CUtensorMap* map)
{
    PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
    const size_t elem = fp64 ? sizeof(double) : sizeof(float);
    if (!encode || base == nullptr || (reinterpret_cast<uintptr_t>(base) & 15) != 0 || (size_t(N) * elem) % 16 != 0)
        return false;
    const cuuint64_t dims[3] = {cuuint64_t(N), cuuint64_t(N), 3};
    const cuuint64_t strides[2] = {cuuint64_t(N) * elem, cuuint64_t(N) * N * elem};
    const cuuint32_t box[3] = {cuuint32_t(cols), 1, 3};
    const cuuint32_t estr[3] = {1, 1, 1};
    return encode(map, fp64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3,
                  const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The two-column sweep's rows arrive by per-lane asynchronous copies (0, the
// default and the faster) or by bulk tensor copies (1).
std::atomic<int> g_sweep_tma{0};

// Launch shape of the single-mesh sweep: warps per block and how many waves
// of resident warps the segments fill (0 = default: 4 warps, 2 waves; two
// waves let the block scheduler refill the slots of early finishers, 1.5%
// faster at 4096^2 than one wave).
std::atomic<int> g_sweep_block_warps{0}, g_sweep_waves{0};

// Rows per warp: enough segments along x that all strips fill `waves` waves
// of resident warps, down to 2 rows (32 with a single wave). Only small and
// medium meshes reach short segments; there filling the GPU with warps
// matters more than the halo rows each segment recomputes (256^2: 1.34 G
// cell-updates/s with 16-row segments, 1.75 G with 8, 2.11 G with 4, 2.23 G
// with 2).
// Resident warps of one sweep instantiation (blocks per SM x warps per block
// x SMs), per device and block size (block_warps is 1, 2 or 4), queried once.
template<int KIND, int COLS, bool DIAG, bool TMA>
int sweep_capacity(int wpb, size_t smem, int dev, int* capacity)
{
    static PerDeviceOnce once[5];
    static int blocks_per_sm[64][5] = {};
    static int sm_count[64][5] = {};
    if (int r = once[wpb].run(dev, [&]() -> int {
            int b = 0, n = 0;
            MARA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, sweep_kernel<KIND, COLS, DIAG, TMA>,
                                                                    wpb * 32, smem));
            MARA_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
            sm_count[dev & 63][wpb] = n;
            blocks_per_sm[dev & 63][wpb] = b > 0 ? b : 1;
            return MARA_OK;
        }))
        return r;
    *capacity = blocks_per_sm[dev & 63][wpb] * wpb * sm_count[dev & 63][wpb];
    return MARA_OK;
}

template<int KIND, int COLS, bool DIAG>
int launch_sweep(Args A, cudaStream_t s)
{
    const int set_wpb = g_sweep_block_warps.load(std::memory_order_relaxed);
    const int set_waves = g_sweep_waves.load(std::memory_order_relaxed);
    const int wpb = set_wpb > 0 ? set_wpb : SW_WARPS;
    const int waves = set_waves > 0 ? set_waves : 2;
    int dev = 0;
    MARA_CUDA(cudaGetDevice(&dev));
    CUtensorMap umap, dmap;
    std::memset(&umap, 0, sizeof umap);
    std::memset(&dmap, 0, sizeof dmap);
    const bool tma = COLS == 2 && g_sweep_tma.load(std::memory_order_relaxed) && row_tensor_map(A.u_in, A.N, true, 64, &umap) &&
                     (KIND != K_MIX2 || row_tensor_map(A.d1, A.N, false, TRING_D_COLS, &dmap));
    const size_t smem = COLS == 2 ? size_t(wpb) * (tma ? TRING_WARP_BYTES : RING_WARP_BYTES) : 0;
    int capacity = 0;
    if (int r = tma ? sweep_capacity<KIND, COLS, DIAG, true>(wpb, smem, dev, &capacity)
                    : sweep_capacity<KIND, COLS, DIAG, false>(wpb, smem, dev, &capacity))
        return r;
    const int cols = COLS == 2 ? SW2_COLS : SW_COLS;
    A.tiles_y = (A.N + cols - 1) / cols;
    const int segments = std::max(1, waves * capacity / A.tiles_y);
    A.sweep_rows = std::max(waves > 1 ? 2 : 32, (A.N + segments - 1) / segments);
    const int strips_x = (A.N + A.sweep_rows - 1) / A.sweep_rows;
    const int warps = strips_x * A.tiles_y;
    const int blocks = (warps + wpb - 1) / wpb + (A.side_binary ? 1 : 0);
    if (tma) sweep_kernel<KIND, COLS, DIAG, true><<<blocks, wpb * 32, smem, s>>>(A, umap, dmap);
    else sweep_kernel<KIND, COLS, DIAG, false><<<blocks, wpb * 32, smem, s>>>(A, umap, dmap);
    return launch_status("minidisk sweep kernel");
}

// Columns per lane of the mixed sweep: 0 = automatic (two wherever the mesh
// and buffers allow), 1 or 2 to force one form.
std::atomic<int> g_sweep_columns{0};

bool two_column_ok(const Args& A)
{
    auto al = [](const void* p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) & (a - 1)) == 0; };
    return A.N % 2 == 0 && al(A.u_in, 16) && al(A.u_out, 16) && al(A.d1, 8) && al(A.d_out, 8);
}

template<int KIND>
int launch_sweep_auto(const Args& A, cudaStream_t s)
{
    const bool two = g_sweep_columns.load(std::memory_order_relaxed) != 1 && two_column_ok(A);
    if (A.diag) return two ? launch_sweep<KIND, 2, true>(A, s) : launch_sweep<KIND, 1, true>(A, s);
    return two ? launch_sweep<KIND, 2, false>(A, s) : launch_sweep<KIND, 1, false>(A, s);
}

// ------------------------------------------------------------- diagnostics (FP64)
// The rate-vector sums 0..12 of a state u (+ the FP32 increment d1) in FP64,
// the source-term fields as problems/minidisk_scheme.cpp:47-76 and
// src/physics_two_body.hpp:200-218 define them. The binary comes from the
// clock row A.stage, or A.bin when A.clock is null.
__global__ void __launch_bounds__(256) rates_kernel(const Args A, const double* u, const float* d1, double* out)
{
    __shared__ double part[DIAG_SUMS][8];
    const int N = A.N;
    const int64_t NN = int64_t(N) * N;
    const double* bin = A.clock ? A.clock->binary[A.stage] : A.bin;
    const double m1 = bin[0], x1 = bin[1], y1 = bin[2], m2 = bin[3], x2 = bin[4], y2 = bin[5];
    double acc[DIAG_SUMS] = {};
    for (int64_t c = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; c < NN; c += int64_t(gridDim.x) * blockDim.x)
    {
        const int i = int(c / N), j = int(c - int64_t(i) * N);
        // cell centres: adjacent_mean of the block's vertex linspace
        const int ki = i % A.n, kj = j % A.n;
        const uint64_t bi = uint64_t(i / A.n), bj = uint64_t(j / A.n);
        const double x = 0.5 * (vertex(A.R, A.n, A.level, bi, ki) + vertex(A.R, A.n, A.level, bi, ki + 1));
        const double y = 0.5 * (vertex(A.R, A.n, A.level, bj, kj) + vertex(A.R, A.n, A.level, bj, kj + 1));
        double w[3];
        for (int k = 0; k < 3; ++k) w[k] = u[k * NN + c] + (d1 ? double(d1[k * NN + c]) : 0.0);
        auto sink = [&](double px, double py) {
            const double dx = x - px, dy = y - py;
            return A.sink_rate * exp(-pow(0.0 + dx * dx + dy * dy, 3.0) / A.s6);
        };
        auto accel = [&](double m, double px, double py, double& ax, double& ay) {
            const double dx = x - px, dy = y - py;
            const double g = -1.0 * m / pow(dx * dx + dy * dy + A.rs2, 1.5);
            ax = g * dx;
            ay = g * dy;
        };
        const double sr1 = sink(x1, y1), sr2 = sink(x2, y2);
        double a1x, a1y, a2x, a2y;
        accel(m1, x1, y1, a1x, a1y);
        accel(m2, x2, y2, a2x, a2y);
        const double rr = sqrt(0.0 + x * x + y * y);
        const double br = 0.5 * A.buffer_rate * (1.0 + tanh((rr - A.R) / A.buffer_scale));
        const double v[DIAG_SUMS] = {
            w[0] * sr1, w[0] * sr2, w[1] * sr1, w[2] * sr1, w[1] * sr2, w[2] * sr2,
            -w[0] * a1x, -w[0] * a1y, -w[0] * a2x, -w[0] * a2y,
            (1.0 - w[0]) * br, w[0], x * w[2] - y * w[1]};
        for (int k = 0; k < DIAG_SUMS; ++k) acc[k] += v[k];
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int k = 0; k < DIAG_SUMS; ++k)
    {
        double v = acc[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) part[k][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < DIAG_SUMS)
    {
        double v = 0.0;
        for (int w = 0; w < int(blockDim.x >> 5); ++w) v += part[threadIdx.x][w];
        atomicAdd(out + threadIdx.x, v * (A.dl * A.dl));
    }
}

// Entries 13..15 of a rate row from its force sums and the binary (position
// and velocity) at the row's time.
__global__ void rates_finish_kernel(double* r, Binary b)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    r[13] = b.x1 * r[7] - b.y1 * r[6];
    r[14] = b.x2 * r[9] - b.y2 * r[8];
    r[15] = (r[6] * b.vx1 + r[7] * b.vy1) + (r[8] * b.vx2 + r[9] * b.vy2);
}

int launch_rates(const Args& A, const double* u, const float* d1, double* out, cudaStream_t s)
{
    const int64_t NN = int64_t(A.N) * A.N;
    const int blocks = int(std::min<int64_t>((NN + 255) / 256, 152 * 8));
    rates_kernel<<<blocks, 256, 0, s>>>(A, u, d1, out);
    return launch_status("minidisk rates_kernel");
}

// ------------------------------------------------------------- clock kernel
__global__ void clock_kernel(mara_minidisk_clock* c, const ClockArgs a)
{
    // two lanes: the stage binaries (FP64 Kepler solves) run side by side
    if (threadIdx.x >= 2 || blockIdx.x != 0) return;
    advance_clock(c, a, int(threadIdx.x), 2);
}

// ------------------------------------------------------------- small kernels
__global__ void initial_kernel(int N, int n, int level, double R, double rs2, double omega,
                               uint64_t seed, double amplitude, double* u)
{
    size_t NN = size_t(N) * N;
    for (size_t c = blockIdx.x * size_t(blockDim.x) + threadIdx.x; c < NN; c += size_t(gridDim.x) * blockDim.x)
    {
        int i = int(c / N), j = int(c % N);
        uint64_t bi = uint64_t(i / n), bj = uint64_t(j / n);
        int ki = i - int(bi) * n, kj = j - int(bj) * n;
        double x = 0.5 * (vertex(R, n, level, bi, ki) + vertex(R, n, level, bi, ki + 1));
        double y = 0.5 * (vertex(R, n, level, bj, kj) + vertex(R, n, level, bj, kj + 1));
        // explicit round-to-nearest operations: bit-identical to the host formulae
        double r2 = __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y));
        double ph = __ddiv_rn(-1.0, __dsqrt_rn(__dadd_rn(r2, rs2)));
        double r0 = __dsqrt_rn(r2);
        double vp = __dadd_rn(__dsqrt_rn(-ph), -__dmul_rn(omega, r0));
        double vx = __dmul_rn(vp, __ddiv_rn(-y, r0));
        double vy = __dmul_rn(vp, __ddiv_rn(x, r0));
        double sig = 1.0;
        if (amplitude != 0.0)
        {
            uint64_t z = seed + (uint64_t(c) + 1) * 0x9E3779B97F4A7C15ull;
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
            z ^= z >> 31;
            double r = __dadd_rn(__dmul_rn(2.0, double(z >> 11) * 0x1.0p-53), -1.0);
            sig = __dmul_rn(sig, __dadd_rn(1.0, __dmul_rn(amplitude, r)));
        }
        vx = __dmul_rn(sig, vx);
        vy = __dmul_rn(sig, vy);
        u[c] = sig;
        u[NN + c] = vx;
        u[2 * NN + c] = vy;
    }
}

// Fastest wavespeed of a state in FP32 (mixed-precision runs): the same
// estimate as the fused reduction of the mixed stage kernels.
// The mixed path's CFL clock init: the FP32 wavespeed of every cell reduced
// to the speed key of the fastest cell (as the stage kernels do), then that
// cell's FP64 wavespeed (key_to_wavespeed_kernel). An FP64 reduction over
// every cell costs FP64 divisions per cell, which GB300 runs slowly.
// With u_copy set, the kernel also copies u into it: the host-buffer call
// reads the caller's pinned state over the host link once, here.
__global__ void wavespeed_key_kernel(int N, FloatConsts F, const double* u, unsigned long long* key_out,
                                     double* u_copy)
{
    __shared__ unsigned long long wk[NT / 32];
    const size_t NN = size_t(N) * N;
    unsigned long long key = 0ull;
    for (size_t c = blockIdx.x * size_t(blockDim.x) + threadIdx.x; c < NN; c += size_t(gridDim.x) * blockDim.x)
    {
        const int i = int(c / N), j = int(c % N);
        const float x = fmaf(float(i) + 0.5f, F.dl, -F.R), y = fmaf(float(j) + 0.5f, F.dl, -F.R);
        const float spot = sqrt_fast(rsqrt_fast(fmaf(x, x, y * y) + F.rs2));
        const double s = u[c], m1 = u[NN + c], m2 = u[2 * NN + c];
        if (u_copy)
        {
            u_copy[c] = s;
            u_copy[NN + c] = m1;
            u_copy[2 * NN + c] = m2;
        }
        key = key_max(key, speed_key(wavespeed_f(F, d2f(s), d2f(m1), d2f(m2), spot), c));
    }
    for (int o = 16; o > 0; o >>= 1) key = key_max(key, __shfl_xor_sync(0xffffffffu, key, o));
    if ((threadIdx.x & 31) == 0) wk[threadIdx.x >> 5] = key;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        unsigned long long r = 0ull;
        for (int w = 0; w < int(blockDim.x / 32); ++w) r = key_max(r, wk[w]);
        atomicMax(key_out, r);
    }
}

__global__ void key_to_wavespeed_kernel(mara_minidisk_clock* clock, const ClockArgs a, const double* u)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const unsigned long long key = __double_as_longlong(clock->max_wavespeed);
    if (key != 0ull)
        clock->max_wavespeed = cell_wavespeed(u, size_t(a.N) * a.N, a.N, a.n, a.level, a.R, a.rs2, a.mach,
                                              size_t(unsigned(key)));
}

// Fastest wavespeed of a state (for the first CFL step), FP64.
__global__ void wavespeed_kernel(int N, int n, int level, double R, double rs2, double mach,
                                 const double* u, unsigned long long* amax)
{
    __shared__ double wm[NT / 32];
    size_t NN = size_t(N) * N;
    double m = 0.0;
    for (size_t c = blockIdx.x * size_t(blockDim.x) + threadIdx.x; c < NN; c += size_t(gridDim.x) * blockDim.x)
        m = fmax(m, cell_wavespeed(u, NN, N, n, level, R, rs2, mach, c));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        double r = 0.0;
        for (int w = 0; w < int(blockDim.x / 32); ++w) r = fmax(r, wm[w]);
        atomicMax(amax, (unsigned long long)__double_as_longlong(r));
    }
}

__global__ void recover_primitive_kernel(const double* u, int64_t count, double* p)
{
    for (int64_t c = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; c < count; c += int64_t(gridDim.x) * blockDim.x)
    {
        double s = u[3 * c], m1 = u[3 * c + 1], m2 = u[3 * c + 2];
        p[3 * c] = s; p[3 * c + 1] = m1 / s; p[3 * c + 2] = m2 / s;
    }
}

__global__ void gradient_kernel(const double* pc, int64_t n0, int64_t n1, int axis, double theta, double* out)
{
    const int64_t m0 = axis == 0 ? n0 - 2 : n0, m1 = axis == 0 ? n1 : n1 - 2;
    const int64_t di = axis == 0 ? 1 : 0, dj = axis == 0 ? 0 : 1;
    for (int64_t c = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; c < m0 * m1 * 3; c += int64_t(gridDim.x) * blockDim.x)
    {
        int64_t k = c % 3, cell = c / 3, i = cell / m1, j = cell % m1;
        double yl = pc[(i * n1 + j) * 3 + k];
        double y0 = pc[((i + di) * n1 + j + dj) * 3 + k];
        double yr = pc[((i + 2 * di) * n1 + j + 2 * dj) * 3 + k];
        out[c] = plm(yl, y0, yr, theta);
    }
}

// ------------------------------------------------------------- host helpers
int check_params(const mara_minidisk_params* sd)
{
    MARA_REQUIRE(sd != nullptr, "minidisk: params is null");
    MARA_REQUIRE(sd->block_size >= 1 && sd->block_size <= (1 << 16), "minidisk: block_size out of range");
    MARA_REQUIRE(sd->depth >= 0 && sd->depth <= 12, "minidisk: depth out of range");
    MARA_REQUIRE(int64_t(sd->block_size) << sd->depth <= 65536, "minidisk: mesh wider than 65536 cells");
    MARA_REQUIRE(sd->mach_number > 0.0, "minidisk: mach_number must be positive");
    MARA_REQUIRE(sd->buffer_scale > 0.0, "minidisk: buffer_scale must be positive");
    MARA_REQUIRE(sd->mass_ratio > 0.0, "minidisk: mass_ratio must be positive");
    MARA_REQUIRE(sd->eccentricity >= 0.0 && sd->eccentricity < 1.0, "minidisk: eccentricity must be in [0, 1)");
    return MARA_OK;
}

inline double cell_size(const mara_minidisk_params* sd, int level)
{
    return 2.0 * sd->domain_radius / double(sd->block_size) / double(1 << level);
}

Args base_args(const mara_minidisk_params* sd)
{
    Args A;
    std::memset(&A, 0, sizeof A);
    A.n = sd->block_size;
    A.level = sd->depth;
    A.N = sd->block_size << sd->depth;
    A.R = sd->domain_radius;
    A.dl = cell_size(sd, sd->depth);
    A.rs2 = std::pow(sd->softening_length, 2.0);
    A.mach = sd->mach_number;
    A.nu = sd->nu;
    A.omega = sd->omega_frame;
    A.mass_ratio = sd->mass_ratio;
    A.eccentricity = sd->eccentricity;
    A.side_binary = 0;
    A.sink_rate = sd->sink_rate;
    A.s6 = std::pow(sd->sink_radius, 6.0);
    A.buffer_rate = sd->buffer_rate;
    A.buffer_scale = sd->buffer_scale;
    A.theta = sd->plm_theta;
    FloatConsts& f = A.f;
    f.rs2 = float(A.rs2);
    f.inv_mach2 = float(1.0 / (A.mach * A.mach));
    f.inv_mach = float(1.0 / A.mach);
    f.half_nu = float(A.nu * 0.5);
    f.half_inv_dl = float(0.5 / A.dl);
    f.quarter_inv_dl = f.half_inv_dl * 0.5f;
    f.inv_dl = float(1.0 / A.dl);
    f.theta = float(A.theta);
    f.two_theta = 2.0f * f.theta;
    f.R = float(A.R);
    f.dl = float(A.dl);
    f.sink_rate = float(A.sink_rate);
    f.inv_s6 = float(1.0 / A.s6);
    f.buffer_rate = float(A.buffer_rate);
    f.neg2_inv_buffer_scale = float(-2.0 / A.buffer_scale);
    f.omega = float(A.omega);
    f.omega2 = float(A.omega * A.omega);
    f.two_omega = float(2.0 * A.omega);
    f.visc_mu = float(A.nu * 0.5 * 0.25 / A.dl);
    f.sink_ex2 = float(-1.4426950408889634 / A.s6);
    f.buffer_ex2 = float(-2.0 * 1.4426950408889634 / A.buffer_scale);
    // q^3 |sink_ex2| >= 127 (after the three roundings of the device's
    // product, still above 126.99): 2^(q^3 sink_ex2) < 2^-126 flushes to zero
    const double c = std::fabs(double(f.sink_ex2));
    f.sink_far = std::isfinite(c) && c > 0.0 ? float(std::cbrt(127.0 / c) * (1.0 + 1e-6)) : INFINITY;
    return A;
}

void set_binary(Args& A, const mara_minidisk_params* sd, double t)
{
    Binary b = binary_state(sd->mass_ratio, sd->eccentricity, sd->omega_frame, t);
    double v[6] = {b.m1, b.x1, b.y1, b.m2, b.x2, b.y2};
    std::memcpy(A.bin, v, sizeof v);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library); null if the driver does not provide it.
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

// The [3][N][N] FP64 state as a 3D tensor with the halo tile's 36 x 20 x 3
// box; false (and the per-thread tile loads) where TMA cannot address it:
// N odd (row stride not a multiple of 16 bytes) or an unaligned state.
bool state_tensor_map(const double* u, int N, CUtensorMap* map)
{
    PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
    if (!encode || N % 2 != 0 || (reinterpret_cast<uintptr_t>(u) & 15) != 0) return false;
    const cuuint64_t dims[3] = {cuuint64_t(N), cuuint64_t(N), 3};
    const cuuint64_t strides[2] = {cuuint64_t(N) * sizeof(double), cuuint64_t(N) * N * sizeof(double)};
    const cuuint32_t box[3] = {EY, EX, 3};
    const cuuint32_t elem[3] = {1, 1, 1};
    return encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<double*>(u), dims, strides, box, elem,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template<typename R, int KIND>
int launch_stage(const Args& A, int tiles, cudaStream_t s)
{
    static PerDeviceOnce once;
    int dev = 0;
    MARA_CUDA(cudaGetDevice(&dev));
    if (int r = once.run(dev, []() -> int {
            MARA_CUDA(cudaFuncSetAttribute(stage_kernel<R, KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           int(sizeof(Smem<R>))));
            return MARA_OK;
        }))
        return r;
    Args a = A;
    CUtensorMap map;
    std::memset(&map, 0, sizeof map);
    a.use_tma = KIND == K_FP64 && A.N >= TX + 4 && state_tensor_map(A.u_in, A.N, &map);
    stage_kernel<R, KIND><<<tiles, NT, sizeof(Smem<R>), s>>>(a, map);
    return launch_status("minidisk stage kernel");
}

int grid_stage(Args A, int kind, cudaStream_t s)
{
    if (A.N >= 64 && kind == K_MIX1) return A.d_out ? launch_sweep_auto<K_MIXD>(A, s) : launch_sweep_auto<K_MIX1>(A, s);
    if (A.N >= 64 && kind == K_MIX2) return launch_sweep_auto<K_MIX2>(A, s);
    if (A.diag)
    {
        // no fused sums outside the mixed sweeps: reduce the stage input first
        if (int r = launch_rates(A, A.u_in, kind == K_MIX2 ? A.d1 : nullptr, A.diag, s)) return r;
        A.diag = nullptr;
    }
    int tiles_x = (A.N + TX - 1) / TX;
    A.tiles_y = (A.N + TY - 1) / TY;
    int tiles = tiles_x * A.tiles_y;
    switch (kind)
    {
        case K_FP64: return launch_stage<double, K_FP64>(A, tiles, s);
        case K_MIX1: return launch_stage<float, K_MIX1>(A, tiles, s);
        case K_MIX2: return launch_stage<float, K_MIX2>(A, tiles, s);
    }
    return fail(MARA_ERR_ARGUMENT, "minidisk: bad stage kind");
}

ClockArgs clock_args(const mara_minidisk_params* sd, int dt_mode, int rk_order, int end_step, int begin_step)
{
    ClockArgs a;
    a.diag = nullptr;
    a.wavespeed_key = 0;
    a.key_state = 0;
    a.u_key[0] = a.u_key[1] = nullptr;
    a.N = sd->block_size << sd->depth;
    a.n = sd->block_size;
    a.level = sd->depth;
    a.rs2 = std::pow(sd->softening_length, 2.0);
    a.mach = sd->mach_number;
    a.R = sd->domain_radius;
    a.dl = cell_size(sd, sd->depth);
    a.cfl = sd->cfl;
    a.softening_length = sd->softening_length;
    a.mass_ratio = sd->mass_ratio;
    a.eccentricity = sd->eccentricity;
    a.omega = sd->omega_frame;
    a.dt_mode = dt_mode;
    a.rk_order = rk_order;
    a.end_step = end_step;
    a.begin_step = begin_step;
    a.binaries = 1;
    return a;
}

int clock_step(const mara_minidisk_params* sd, mara_minidisk_clock* clock, int dt_mode, int rk_order,
               int end_step, int begin_step, cudaStream_t s, mara_minidisk_diagnostics* diag = nullptr,
               const double* key_state = nullptr, int binaries = 1)
{
    ClockArgs a = clock_args(sd, dt_mode, rk_order, end_step, begin_step);
    a.diag = diag;
    a.binaries = binaries;
    if (key_state)
    {
        a.wavespeed_key = 1;
        a.u_key[0] = key_state;
    }
    clock_kernel<<<1, 32, 0, s>>>(clock, a);
    return launch_status("minidisk clock kernel");
}

} // namespace md
} // namespace mara

using namespace mara;
using namespace mara::md;

extern "C" {

int mara_minidisk_binary(const mara_minidisk_params* sd, double time, double* out)
{
    if (int r = check_params(sd)) return r;
    MARA_REQUIRE(out != nullptr, "mara_minidisk_binary: out is null");
    Binary b = binary_state(sd->mass_ratio, sd->eccentricity, sd->omega_frame, time);
    double v[10] = {b.m1, b.x1, b.y1, b.vx1, b.vy1, b.m2, b.x2, b.y2, b.vx2, b.vy2};
    std::memcpy(out, v, sizeof v);
    return MARA_OK;
}

int mara_minidisk_dt_formula(const mara_minidisk_params* sd, double time, double* dt)
{
    if (int r = check_params(sd)) return r;
    MARA_REQUIRE(dt != nullptr, "mara_minidisk_dt_formula: dt is null");
    double dx = 2.0 * sd->domain_radius / double(sd->block_size) / double(1 << sd->depth);
    double vmax = std::sqrt(1.0 * 0.5 / sd->softening_length);
    double cfl = sd->cfl * std::min(1.0, 0.01 + time / 0.05);
    *dt = dx / vmax * cfl;
    return MARA_OK;
}

int mara_minidisk_updated_conserved(const mara_minidisk_params* sd, const double* uc, const double* pe,
                                    double time, double dt, uint32_t level, uint64_t bi, uint64_t bj,
                                    double* u1, void* stream)
{
    if (int r = check_params(sd)) return r;
    MARA_REQUIRE(uc && pe && u1, "mara_minidisk_updated_conserved: null buffer");
    MARA_REQUIRE(level <= 30 && bi < (uint64_t(1) << level) && bj < (uint64_t(1) << level),
                 "mara_minidisk_updated_conserved: block index outside its level");
    Args A = base_args(sd);
    A.level = int(level);
    A.N = sd->block_size;
    A.dl = cell_size(sd, int(level));
    A.bi = bi;
    A.bj = bj;
    A.dt = dt;
    set_binary(A, sd, time);
    A.u_in = uc;
    A.pe = pe;
    A.u_out = u1;
    int tiles_x = (A.n + TX - 1) / TX;
    A.tiles_y = (A.n + TY - 1) / TY;
    return launch_stage<double, K_BLOCK>(A, tiles_x * A.tiles_y, as_stream(stream));
}

int mara_minidisk_recover_primitive(const double* u, int64_t count, double* p, void* stream)
{
    MARA_REQUIRE(count >= 0, "mara_minidisk_recover_primitive: negative count");
    if (count == 0) return MARA_OK;
    MARA_REQUIRE(u && p, "mara_minidisk_recover_primitive: null buffer");
    int blocks = int(std::min<int64_t>((count + 255) / 256, 152 * 16));
    recover_primitive_kernel<<<blocks, 256, 0, as_stream(stream)>>>(u, count, p);
    return launch_status("recover_primitive_kernel");
}

int mara_minidisk_estimate_gradient(const double* pc, int64_t n0, int64_t n1, int32_t axis, double theta,
                                    double* out, void* stream)
{
    MARA_REQUIRE(axis == 0 || axis == 1, "mara_minidisk_estimate_gradient: axis must be 0 or 1");
    MARA_REQUIRE((axis == 0 ? n0 : n1) >= 2 && n0 >= 0 && n1 >= 0, "mara_minidisk_estimate_gradient: array too small");
    int64_t total = (axis == 0 ? (n0 - 2) * n1 : n0 * (n1 - 2)) * 3;
    if (total == 0) return MARA_OK;
    MARA_REQUIRE(pc && out, "mara_minidisk_estimate_gradient: null buffer");
    int blocks = int(std::min<int64_t>((total + 255) / 256, 152 * 16));
    gradient_kernel<<<blocks, 256, 0, as_stream(stream)>>>(pc, n0, n1, axis, theta, out);
    return launch_status("gradient_kernel");
}

int mara_minidisk_substep(const mara_minidisk_params* sd, const double* u_in, const double* u_avg, double* u_out,
                          double time, double dt, void* stream)
{
    if (int r = check_params(sd)) return r;
    MARA_REQUIRE(u_in && u_out, "mara_minidisk_substep: null buffer");
    MARA_REQUIRE(u_in != u_out, "mara_minidisk_substep: u_out must not alias u_in");
    Args A = base_args(sd);
    A.dt = dt;
    set_binary(A, sd, time);
    A.u_in = u_in;
    A.u_avg = u_avg;
    A.u_out = u_out;
    return grid_stage(A, K_FP64, as_stream(stream));
}

int mara_minidisk_initial_conserved(const mara_minidisk_params* sd, uint64_t seed, double amplitude,
                                    double* u, void* stream)
{
    if (int r = check_params(sd)) return r;
    MARA_REQUIRE(u != nullptr, "mara_minidisk_initial_conserved: u is null");
    int N = sd->block_size << sd->depth;
    int64_t NN = int64_t(N) * N;
    int blocks = int(std::min<int64_t>((NN + 255) / 256, 152 * 32));
    initial_kernel<<<blocks, 256, 0, as_stream(stream)>>>(N, sd->block_size, sd->depth, sd->domain_radius,
        std::pow(sd->softening_length, 2.0), sd->omega_frame, seed, amplitude, u);
    return launch_status("initial_kernel");
}

int64_t mara_minidisk_workspace_bytes(const mara_minidisk_params* sd, int32_t rk_order, int32_t precision)
{
    if (check_params(sd)) return -1;
    int64_t NN = int64_t(sd->block_size << sd->depth) * (sd->block_size << sd->depth);
    int64_t state = 3 * NN * int64_t(sizeof(double));
    // mixed RK2: the FP32 stage-1 increment and 64 bytes for the next step's
    // stage-1 binary (solved during stage 1, moved into the clock by stage 2)
    if (precision == MARA_MIXED && rk_order == 2) return state + 3 * NN * int64_t(sizeof(float)) + kNextBinaryBytes;
    return state;
}

} // extern "C"

namespace mara {
namespace md {

// u_copy (mixed precision only): also copy u there, and take the fastest
// cell's FP64 wavespeed from the copy.
int clock_init(const mara_minidisk_params* sd, const double* u, double time, mara_minidisk_clock* clock,
               int precision, cudaStream_t s, double* u_copy)
{
    mara_minidisk_clock c;
    std::memset(&c, 0, sizeof c);
    c.time = time;
    // The host value lives on this stack frame: copy synchronously w.r.t. the host.
    MARA_CUDA(cudaMemcpyAsync(clock, &c, sizeof c, cudaMemcpyHostToDevice, s));
    MARA_CUDA(cudaStreamSynchronize(s));
    const int N = sd->block_size << sd->depth;
    const int64_t NN = int64_t(N) * N;
    const int blocks = int(std::min<int64_t>((NN + 255) / 256, 152 * 8));
    auto* amax = reinterpret_cast<unsigned long long*>(&clock->max_wavespeed);
    if (precision == MARA_MIXED)
    {
        // the CFL dt stays an FP64 quantity: the fastest cell's FP64 wavespeed
        wavespeed_key_kernel<<<blocks, NT, 0, s>>>(N, base_args(sd).f, u, amax, u_copy);
        if (int r = launch_status("wavespeed_key_kernel")) return r;
        key_to_wavespeed_kernel<<<1, 32, 0, s>>>(clock, clock_args(sd, MARA_DT_CFL, 2, 0, 0), u_copy ? u_copy : u);
        return launch_status("key_to_wavespeed_kernel");
    }
    wavespeed_kernel<<<blocks, NT, 0, s>>>(N, sd->block_size, sd->depth, sd->domain_radius,
        std::pow(sd->softening_length, 2.0), sd->mach_number, u, amax);
    return launch_status("wavespeed_kernel");
}

} // namespace md
} // namespace mara

extern "C" {

int mara_minidisk_clock_init(const mara_minidisk_params* sd, const double* u, double time,
                             mara_minidisk_clock* clock, void* stream)
{
    if (int r = check_params(sd)) return r;
    MARA_REQUIRE(u && clock, "mara_minidisk_clock_init: null buffer");
    return clock_init(sd, u, time, clock, MARA_FP64, as_stream(stream));
}

int mara_minidisk_advance(const mara_minidisk_params* sd, double* u, mara_minidisk_clock* clock,
                          int32_t steps, int32_t rk_order, int32_t precision, int32_t dt_mode,
                          void* workspace, void* stream)
{
    return mara_minidisk_advance_diag(sd, u, clock, steps, rk_order, precision, dt_mode, workspace, nullptr, stream);
}

int mara_minidisk_advance_diag(const mara_minidisk_params* sd, double* u, mara_minidisk_clock* clock,
                               int32_t steps, int32_t rk_order, int32_t precision, int32_t dt_mode,
                               void* workspace, mara_minidisk_diagnostics* diag, void* stream)
{
    return advance_impl(sd, u, clock, steps, rk_order, precision, dt_mode, workspace, diag, stream, nullptr);
}

} // extern "C"

namespace mara {
namespace md {

// The advance loop. final_out (mixed RK2 only): the last step's second stage
// writes the new state there instead of u, which is then left at the state
// before that step; the host-buffer call passes the caller's pinned output.
int advance_impl(const mara_minidisk_params* sd, double* u, mara_minidisk_clock* clock, int32_t steps,
                 int32_t rk_order, int32_t precision, int32_t dt_mode, void* workspace,
                 mara_minidisk_diagnostics* diag, void* stream, double* final_out)
{
    if (int r = check_params(sd)) return r;
    MARA_REQUIRE(u && clock && workspace, "mara_minidisk_advance: null buffer");
    MARA_REQUIRE(steps >= 0, "mara_minidisk_advance: negative step count");
    MARA_REQUIRE(rk_order == 1 || rk_order == 2, "mara_minidisk_advance: rk_order must be 1 or 2");
    MARA_REQUIRE(precision == MARA_FP64 || precision == MARA_MIXED, "mara_minidisk_advance: bad precision");
    MARA_REQUIRE(dt_mode >= MARA_DT_FORMULA && dt_mode <= MARA_DT_FORMULA_HELD, "mara_minidisk_advance: bad dt_mode");
    if (steps == 0) return MARA_OK;
    cudaStream_t s = as_stream(stream);
    const int N = sd->block_size << sd->depth;
    const size_t NN = size_t(N) * N;
    double* ws_state = static_cast<double*>(workspace);
    float* ws_d1 = reinterpret_cast<float*>(ws_state + 3 * NN);
    double* ws_next_binary = reinterpret_cast<double*>(ws_d1 + 3 * NN);   // 36 NN bytes in: 8-byte aligned
    unsigned long long* amax = dt_mode == MARA_DT_CFL ? reinterpret_cast<unsigned long long*>(&clock->max_wavespeed) : nullptr;

    Args A = base_args(sd);
    A.clock = clock;
    double* cur = u;
    double* alt = ws_state;

    double* rate0 = diag ? diag->rate[0] : nullptr;
    double* rate1 = diag ? diag->rate[1] : nullptr;
    // mixed RK2 on the sweep path: the stage binaries are solved inside the
    // sweeps (Args::side_binary), off the step's critical path
    const bool side_binaries = precision == MARA_MIXED && rk_order == 2 && N >= 64;

    // a held formula dt is chosen by the call's first step
    if (int r = clock_step(sd, clock, dt_mode == MARA_DT_FORMULA_HELD ? MARA_DT_FORMULA : dt_mode, rk_order, 0, 1, s,
                           diag))
        return r;
    for (int step = 0; step < steps; ++step)
    {
        if (precision == MARA_FP64 && rk_order == 2)
        {
            Args a1 = A; a1.stage = 0; a1.u_in = cur; a1.u_out = ws_state; a1.diag = rate0;
            if (int r = grid_stage(a1, K_FP64, s)) return r;
            Args a2 = A; a2.stage = 1; a2.u_in = ws_state; a2.u_avg = cur; a2.u_out = cur; a2.amax = amax;
            a2.diag = rate1;
            if (int r = grid_stage(a2, K_FP64, s)) return r;
        }
        else if (precision == MARA_FP64)
        {
            Args a1 = A; a1.stage = 0; a1.u_in = cur; a1.u_out = alt; a1.amax = amax; a1.diag = rate0;
            if (int r = grid_stage(a1, K_FP64, s)) return r;
            std::swap(cur, alt);
        }
        else if (rk_order == 2)
        {
            // the sweeps (N >= 64) solve the stage binaries in their block 0
            Args a1 = A; a1.stage = 0; a1.u_in = cur; a1.d_out = ws_d1; a1.diag = rate0;
            a1.side_binary = side_binaries ? 1 : 0;
            a1.next_binary = ws_next_binary;
            if (int r = grid_stage(a1, K_MIX1, s)) return r;
            const bool last_out = final_out && step + 1 == steps;
            Args a2 = A; a2.stage = 1; a2.u_in = cur; a2.d1 = ws_d1; a2.u_out = last_out ? final_out : alt;
            a2.amax = amax;
            a2.amax_key = 1;
            a2.diag = rate1;
            a2.side_binary = side_binaries ? 2 : 0;
            a2.next_binary = ws_next_binary;
            if (int r = grid_stage(a2, K_MIX2, s)) return r;
            if (last_out) cur = final_out;
            else std::swap(cur, alt);
        }
        else
        {
            Args a1 = A; a1.stage = 0; a1.u_in = cur; a1.u_out = alt; a1.amax = amax; a1.diag = rate0;
            a1.amax_key = 1;
            if (int r = grid_stage(a1, K_MIX1, s)) return r;
            std::swap(cur, alt);
        }
        // mixed CFL: the reduction named the fastest cell of the new state cur
        const double* key_state = precision == MARA_MIXED && amax ? cur : nullptr;
        if (int r = clock_step(sd, clock, dt_mode, rk_order, 1, step + 1 < steps, s, diag, key_state,
                               side_binaries ? 0 : 1))
            return r;
    }
    if (cur != u && cur != final_out)
        MARA_CUDA(cudaMemcpyAsync(u, cur, 3 * NN * sizeof(double), cudaMemcpyDeviceToDevice, s));
    return MARA_OK;
}

// The device address of a pinned (page-locked or registered) host buffer, or
// null for any other memory.
const void* pinned_device_address(const void* p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess)
    {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

} // namespace md
} // namespace mara

extern "C" {

int64_t mara_minidisk_host_workspace_bytes(const mara_minidisk_params* sd, int32_t rk_order, int32_t precision)
{
    int64_t ws = mara_minidisk_workspace_bytes(sd, rk_order, precision);
    if (ws < 0) return ws;
    int64_t NN = int64_t(sd->block_size << sd->depth) * (sd->block_size << sd->depth);
    return ws + 3 * NN * int64_t(sizeof(double)) + 256;
}

int mara_minidisk_advance_host(const mara_minidisk_params* sd, const double* u_in, double* u_out, double time,
                               int32_t steps, int32_t rk_order, int32_t precision, int32_t dt_mode,
                               double* time_out, void* workspace, void* stream)
{
    if (int r = check_params(sd)) return r;
    MARA_REQUIRE(u_in && u_out && workspace, "mara_minidisk_advance_host: null buffer");
    cudaStream_t s = as_stream(stream);
    const int N = sd->block_size << sd->depth;
    const size_t bytes = 3 * size_t(N) * N * sizeof(double);
    char* base = static_cast<char*>(workspace);
    double* u = reinterpret_cast<double*>(base);
    auto* clock = reinterpret_cast<mara_minidisk_clock*>(base + bytes);
    void* ws = base + bytes + 256;
    // Mixed RK2 with pinned host buffers: the clock init reads the caller's
    // state over the host link while copying it to the device, and the last
    // stage writes the result straight into the caller's output, so each
    // transfer overlaps a kernel instead of following it.
    const double* in_dev = precision == MARA_MIXED && rk_order == 2 && steps > 0
                         ? static_cast<const double*>(pinned_device_address(u_in)) : nullptr;
    double* out_dev = in_dev ? static_cast<double*>(const_cast<void*>(pinned_device_address(u_out))) : nullptr;
    if (in_dev && out_dev)
    {
        if (int r = clock_init(sd, in_dev, time, clock, precision, s, u)) return r;
        if (int r = advance_impl(sd, u, clock, steps, rk_order, precision, dt_mode, ws, nullptr, stream, out_dev))
            return r;
    }
    else
    {
        MARA_CUDA(cudaMemcpyAsync(u, u_in, bytes, cudaMemcpyHostToDevice, s));
        if (int r = clock_init(sd, u, time, clock, precision, s)) return r;
        if (int r = mara_minidisk_advance(sd, u, clock, steps, rk_order, precision, dt_mode, ws, stream)) return r;
        MARA_CUDA(cudaMemcpyAsync(u_out, u, bytes, cudaMemcpyDeviceToHost, s));
    }
    mara_minidisk_clock c;
    MARA_CUDA(cudaMemcpyAsync(&c, clock, sizeof c, cudaMemcpyDeviceToHost, s));
    MARA_CUDA(cudaStreamSynchronize(s));
    if (time_out) *time_out = c.time;
    return MARA_OK;
}

int mara_minidisk_stage(const mara_minidisk_params* sd, int32_t kind, const double* u_in, const float* d1,
                        const double* u_avg, double* u_out, float* d_out, mara_minidisk_clock* clock,
                        int32_t stage, int32_t reduce_wavespeed, void* stream)
{
    if (int r = check_params(sd)) return r;
    MARA_REQUIRE(kind >= 0 && kind <= 2, "mara_minidisk_stage: kind must be 0, 1 or 2");
    MARA_REQUIRE(stage == 0 || stage == 1, "mara_minidisk_stage: stage must be 0 or 1");
    MARA_REQUIRE(u_in && clock, "mara_minidisk_stage: null buffer");
    MARA_REQUIRE(kind != 2 || (d1 && u_out), "mara_minidisk_stage: kind 2 needs d1 and u_out");
    MARA_REQUIRE(kind != 1 || d_out || u_out, "mara_minidisk_stage: kind 1 needs d_out or u_out");
    MARA_REQUIRE(kind != 0 || u_out, "mara_minidisk_stage: kind 0 needs u_out");
    MARA_REQUIRE(u_out != u_in, "mara_minidisk_stage: u_out must not alias u_in");
    Args A = base_args(sd);
    A.clock = clock;
    A.stage = stage;
    A.u_in = u_in;
    A.d1 = d1;
    A.u_avg = kind == 0 ? u_avg : nullptr;
    A.u_out = u_out;
    A.d_out = kind == 1 ? d_out : nullptr;
    bool writes_state = !(kind == 1 && d_out);
    A.amax = reduce_wavespeed && writes_state ? reinterpret_cast<unsigned long long*>(&clock->max_wavespeed) : nullptr;
    return grid_stage(A, kind == 0 ? K_FP64 : (kind == 1 ? K_MIX1 : K_MIX2), as_stream(stream));
}

int mara_minidisk_sweep_tma(int32_t enable)
{
    if (enable != 0 && enable != 1)
    {
        fail(MARA_ERR_ARGUMENT, "mara_minidisk_sweep_tma: enable must be 0 or 1");
        return -1;
    }
    return g_sweep_tma.exchange(enable);
}

int mara_minidisk_sweep_columns(int32_t columns)
{
    if (columns < 0 || columns > 2)
    {
        fail(MARA_ERR_ARGUMENT, "mara_minidisk_sweep_columns: columns must be 0, 1 or 2");
        return -1;
    }
    return g_sweep_columns.exchange(columns);
}

int mara_minidisk_sweep_shape(int32_t block_warps, int32_t waves)
{
    if (!(block_warps == 0 || block_warps == 1 || block_warps == 2 || block_warps == 4) || waves < 0 || waves > 16)
    {
        fail(MARA_ERR_ARGUMENT, "mara_minidisk_sweep_shape: block_warps must be 0, 1, 2 or 4 and waves in [0, 16]");
        return -1;
    }
    g_sweep_block_warps.store(block_warps);
    g_sweep_waves.store(waves);
    return 0;
}

int mara_minidisk_clock_update(const mara_minidisk_params* sd, mara_minidisk_clock* clock, int32_t dt_mode,
                               int32_t rk_order, int32_t end_step, int32_t begin_step, void* stream)
{
    if (int r = check_params(sd)) return r;
    MARA_REQUIRE(clock != nullptr, "mara_minidisk_clock_update: clock is null");
    MARA_REQUIRE(rk_order == 1 || rk_order == 2, "mara_minidisk_clock_update: rk_order must be 1 or 2");
    MARA_REQUIRE(dt_mode >= MARA_DT_FORMULA && dt_mode <= MARA_DT_FORMULA_HELD, "mara_minidisk_clock_update: bad dt_mode");
    return clock_step(sd, clock, dt_mode, rk_order, end_step != 0, begin_step != 0, as_stream(stream));
}

int mara_minidisk_diagnostics_reset(mara_minidisk_diagnostics* diag, void* stream)
{
    MARA_REQUIRE(diag != nullptr, "mara_minidisk_diagnostics_reset: diag is null");
    MARA_CUDA(cudaMemsetAsync(diag, 0, sizeof *diag, as_stream(stream)));
    return MARA_OK;
}

int mara_minidisk_rates(const mara_minidisk_params* sd, const double* u, const float* d1, double time,
                        double* out, void* stream)
{
    if (int r = check_params(sd)) return r;
    MARA_REQUIRE(u && out, "mara_minidisk_rates: null buffer");
    cudaStream_t s = as_stream(stream);
    Args A = base_args(sd);
    set_binary(A, sd, time);
    MARA_CUDA(cudaMemsetAsync(out, 0, MARA_DIAG_COUNT * sizeof(double), s));
    if (int r = launch_rates(A, u, d1, out, s)) return r;
    rates_finish_kernel<<<1, 32, 0, s>>>(out, binary_state(sd->mass_ratio, sd->eccentricity, sd->omega_frame, time));
    return launch_status("minidisk rates_finish_kernel");
}

} // extern "C"

// ------------------------------------------------------------- allocation-free advance
// Some callers cannot allocate device memory for a workspace: a host program
// that has handed all of the GPU's memory to its own pool allocator, or a
// plugin that only ever receives the caller's state and clock buffers through
// the C ABI and has no allocator of its own to call. For them the scratch of
// mara_minidisk_advance lives in this file-scope device array instead. It is
// sized for meshes of at most MARA_MINIDISK_NOALLOC_MAX_CELLS cells (36 bytes
// per cell: one FP64 state buffer plus the FP32 RK2 increment), and every GPU
// that loads the library holds it until the process exits.
namespace {

constexpr int64_t kNoAllocBytesPerCell = 3 * (sizeof(double) + sizeof(float));
static __device__ __align__(256) unsigned char
    g_noalloc_scratch[MARA_MINIDISK_NOALLOC_MAX_CELLS * kNoAllocBytesPerCell + kNextBinaryBytes];

std::mutex g_noalloc_mutex;
void* g_noalloc_address[64] = {};

// Device address of g_noalloc_scratch on the current device, looked up once
// per device (with that device current). In host code the symbol itself is
// only a host-side stand-in and must never be passed to a kernel.
int noalloc_scratch(void** out)
{
    int dev = 0;
    MARA_CUDA(cudaGetDevice(&dev));
    MARA_REQUIRE(dev >= 0 && dev < 64, "mara_minidisk_advance_noalloc: device index above 63");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (g_noalloc_address[dev] == nullptr)
    {
        void* p = nullptr;
        MARA_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_address[dev] = p;
    }
    *out = g_noalloc_address[dev];
    return MARA_OK;
}

} // namespace

extern "C" int mara_minidisk_advance_noalloc(const mara_minidisk_params* sd, double* u, mara_minidisk_clock* clock,
                                             int32_t steps, int32_t rk_order, int32_t precision, int32_t dt_mode,
                                             void* stream)
{
    if (int r = check_params(sd)) return r;
    const int64_t cells = int64_t(sd->block_size << sd->depth) * int64_t(sd->block_size << sd->depth);
    if (cells > MARA_MINIDISK_NOALLOC_MAX_CELLS)
        return fail(MARA_ERR_ARGUMENT, "mara_minidisk_advance_noalloc: mesh of " + std::to_string(cells) +
                    " cells exceeds the static scratch limit of " + std::to_string(MARA_MINIDISK_NOALLOC_MAX_CELLS) +
                    " cells (use mara_minidisk_advance with a caller-owned workspace)");
    const int64_t need = mara_minidisk_workspace_bytes(sd, rk_order, precision);
    MARA_REQUIRE(need >= 0 && need <= int64_t(sizeof(g_noalloc_scratch)),
                 "mara_minidisk_advance_noalloc: workspace larger than the static scratch");
    void* scratch = nullptr;
    if (int r = noalloc_scratch(&scratch)) return r;
    return mara_minidisk_advance(sd, u, clock, steps, rk_order, precision, dt_mode, scratch, stream);
}
