// Special-relativistic hydrodynamics: conserved -> primitive recovery.
//
// srhd::recover_primitive (src/physics_srhd.hpp:231-285): Newton iteration on
// the pressure, at most 50+1 iterations, converged when |f| < 1e-12 (or
// < 1e-8 on the last iteration), starting from p = 0. One thread per zone;
// zones are read with a (component stride, zone stride) pair so that both the
// GPU's SoA layout and the reference's AoS tuples are accepted.
//
// The default-guess path is written with explicit round-to-nearest
// intrinsics (__dadd_rn, __dmul_rn, __ddiv_rn, __dsqrt_rn) in the reference's
// evaluation order, so no multiply-add is fused and every zone reproduces the
// reference's FP64 result bit for bit.
//
// The learned path (mlp != nullptr) seeds Newton with the pressure predicted
// by a 4-64-64-1 MLP evaluated in BF16 on the tensor cores (see srhd_mlp.cu);
// the same Newton loop and stopping rule then polish in FP64. A zone that
// does not converge within the seeded budget restarts from p = 0 with the
// reference's full budget, so the guess changes the iteration count only.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include "common.cuh"
#include "srhd_mlp.cuh"
#include "srhd_physics.cuh"

namespace mara {
namespace srhd {

struct C2PArgs
{
    const double* cons;
    double* prim;
    int64_t n, cs, zs;           // zone count, component stride, zone stride
    double gamma, floor;
    int32_t* iterations;
    int32_t* status;
    unsigned long long* failures;   // nullable: count of failed zones
    const mlp::Weights* mlp;        // nullable
    int refine32;                   // FP32 Newton iterations applied to the guess
    int seeded_budget;              // FP64 Newton iterations allowed from the guess
};

__device__ inline void store(const C2PArgs& a, int64_t i, const double prim[5], int it, int st)
{
    double* o = a.prim + i * a.zs;
    for (int k = 0; k < 5; ++k) o[k * a.cs] = st == 0 ? prim[k] : 0.0;
    if (a.iterations) a.iterations[i] = it;
    if (a.status) a.status[i] = st;
    if (st != 0 && a.failures) atomicAdd(a.failures, 1ull);
}

__device__ inline Zone load_zone(const C2PArgs& a, int64_t i)
{
    const double* c = a.cons + i * a.zs;
    return Zone{c[0], c[a.cs], c[2 * a.cs], c[3 * a.cs], c[4 * a.cs]};
}

// The reference's recovery from p = 0 of every zone, bit for bit. Each
// thread runs its zone's first kFirstDefault iterations (all but about one
// zone in a hundred converge within them); a zone still iterating waits in a
// per-CTA queue (zone, pressure, iteration count) and resumes later with
// blockDim.x queued zones at a time, so the slow zones (up to the 51
// iterations of the budget) finish in full warps instead of holding up warps
// of converged zones. Resuming gives the same iterates.
constexpr int kFirstDefault = 6;
constexpr int kDefaultThreads = 256;

__global__ void __launch_bounds__(kDefaultThreads) c2p_default_kernel(const C2PArgs a)
{
    __shared__ int64_t q_zone[2 * kDefaultThreads];
    __shared__ double q_p[2 * kDefaultThreads];
    __shared__ int q_it[2 * kDefaultThreads];
    __shared__ int q_n;
    if (threadIdx.x == 0) q_n = 0;
    auto finish = [&](int64_t i, const Zone& z, double p, double W0, bool found, int it) {
        double prim[5] = {0, 0, 0, 0, 0};
        int iters = 0;
        const int st = newton_finish(z, a.floor, p, W0, found, it, prim, iters);
        store(a, i, prim, iters, st);
    };
    auto drain = [&](int from, int count) {
        for (int t = threadIdx.x; t < count; t += blockDim.x)
        {
            const int e = from + t;
            const int64_t i = q_zone[e];
            const Zone z = load_zone(a, i);
            double p = q_p[e], W0 = 1.0;
            int it = q_it[e];
            const bool found = newton_steps(z, a.gamma, p, it, 50, 51, W0);
            finish(i, z, p, W0, found, it);
        }
    };
    for (int64_t base = int64_t(blockIdx.x) * blockDim.x; base < a.n; base += int64_t(gridDim.x) * blockDim.x)
    {
        __syncthreads();
        const int64_t i = base + threadIdx.x;
        if (i < a.n)
        {
            const Zone z = load_zone(a, i);
            double p = 0.0, W0 = 1.0;
            int it = 0;
            const bool found = newton_steps(z, a.gamma, p, it, 50, kFirstDefault, W0);
            if (found || it > 50)
                finish(i, z, p, W0, found, it);
            else
            {
                const int e = atomicAdd(&q_n, 1);
                q_zone[e] = i;
                q_p[e] = p;
                q_it[e] = it;
            }
        }
        __syncthreads();
        const int queued = q_n;
        if (queued >= int(blockDim.x))
        {
            drain(queued - int(blockDim.x), int(blockDim.x));
            __syncthreads();
            if (threadIdx.x == 0) q_n = queued - int(blockDim.x);
        }
    }
    __syncthreads();
    drain(0, q_n);
}

__device__ inline void polish(const C2PArgs& a, int64_t i, const Zone& z, double guess)
{
    if (a.refine32 > 0) guess = refine_fp32(z, a.gamma, guess, a.refine32);
    double prim[5] = {0, 0, 0, 0, 0};
    int it = 0, it2 = 0;
    int st = newton_fast(z, a.gamma, a.floor, guess, a.seeded_budget, prim, it);
    if (st != 0)
    {
        // fall back to the reference's start, budget and arithmetic
        st = newton(z, a.gamma, a.floor, 0.0, 50, prim, it2);
        it += it2;
    }
    store(a, i, prim, it, st);
}

// No network: start from p = 0, sharpen in FP32, polish in FP64.
__global__ void c2p_refined_kernel(const C2PArgs a)
{
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < a.n; i += int64_t(gridDim.x) * blockDim.x)
    {
        const double* c = a.cons + i * a.zs;
        Zone z{c[0], c[a.cs], c[2 * a.cs], c[3 * a.cs], c[4 * a.cs]};
        polish(a, i, z, 0.0);
    }
}

// The end of a seeded polish: primitives from the converged iteration, or the
// fall-back to the reference's start, budget and arithmetic.
__device__ inline void finish_seeded(const C2PArgs& a, int64_t i, const Zone& z, double p, double W0, bool found,
                                     int it)
{
    double prim[5] = {0, 0, 0, 0, 0};
    int iters = 0, it2 = 0;
    int st = newton_fast_finish(z, a.floor, p, W0, found, it, prim, iters);
    if (st != 0)
    {
        st = newton(z, a.gamma, a.floor, 0.0, 50, prim, it2);
        iters += it2;
    }
    store(a, i, prim, iters, st);
}

// Learned guess: the MLP predicts p for kZones zones per CTA (srhd_mlp.cuh),
// then each thread polishes its zone for up to kFirstPolish iterations. A
// zone still short of the stopping rule waits in a per-CTA queue (its zone,
// pressure and iteration count) and resumes later with kThreads queued
// zones at a time, so the few slow zones finish in full warps instead of
// holding a warp of converged zones for the rest of their budget. Resuming
// gives the same iterates, so the result does not depend on the queue.
constexpr int kFirstPolish = 3;

__global__ void __launch_bounds__(mlp::kThreads) c2p_mlp_kernel(const C2PArgs a)
{
    __shared__ mlp::Shared sm;
    __shared__ int64_t q_zone[2 * mlp::kZones];
    __shared__ double q_p[2 * mlp::kZones];
    __shared__ int q_it[2 * mlp::kZones];
    __shared__ int q_n;
    if (threadIdx.x == 0) q_n = 0;
    mlp::begin(*a.mlp, sm);
    // resume queue entries [from, from + count) with one thread each
    auto drain = [&](int from, int count) {
        for (int t = threadIdx.x; t < count; t += blockDim.x)
        {
            const int e = from + t;
            const int64_t i = q_zone[e];
            const Zone z = load_zone(a, i);
            double p = q_p[e], W0 = 1.0;
            int it = q_it[e];
            const bool found = newton_fast_steps(z, a.gamma, p, it, a.seeded_budget, a.seeded_budget + 1, W0);
            finish_seeded(a, i, z, p, W0, found, it);
        }
    };
    uint32_t phase = 0;
    for (int64_t base = int64_t(blockIdx.x) * mlp::kZones; base < a.n; base += int64_t(gridDim.x) * mlp::kZones)
    {
        __syncthreads();
        for (int t = threadIdx.x; t < mlp::kZones; t += blockDim.x)
        {
            int64_t i = base + t;
            float feat[4] = {0.f, 0.f, 0.f, 0.f};
            if (i < a.n)
            {
                const double* c = a.cons + i * a.zs;
                mlp::features(c[0], c[a.cs], c[2 * a.cs], c[3 * a.cs], c[4 * a.cs], feat);
            }
            mlp::stage_features(sm, t, feat);
        }
        __syncthreads();
        mlp::forward(sm, phase);
        __syncthreads();
        for (int t = threadIdx.x; t < mlp::kZones; t += blockDim.x)
        {
            int64_t i = base + t;
            if (i >= a.n) continue;
            const Zone z = load_zone(a, i);
            double guess = mlp::pressure_from_output(sm.out[t], z.D, z.S1, z.S2, z.S3, z.tau);
            if (a.refine32 > 0) guess = refine_fp32(z, a.gamma, guess, a.refine32);
            double p = guess, W0 = 1.0;
            int it = 0;
            const bool found = newton_fast_steps(z, a.gamma, p, it, a.seeded_budget, kFirstPolish, W0);
            if (found || it > a.seeded_budget)
                finish_seeded(a, i, z, p, W0, found, it);
            else
            {
                const int e = atomicAdd(&q_n, 1);
                q_zone[e] = i;
                q_p[e] = p;
                q_it[e] = it;
            }
        }
        __syncthreads();
        const int queued = q_n;
        if (queued >= int(blockDim.x))
        {
            drain(queued - int(blockDim.x), int(blockDim.x));
            __syncthreads();
            if (threadIdx.x == 0) q_n = queued - int(blockDim.x);
        }
    }
    __syncthreads();
    drain(0, q_n);
    mlp::end(sm);
}

__device__ inline double uniform01(uint64_t seed, uint64_t i)
{
    uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return double(z >> 11) * 0x1.0p-53;
}

// Seeded zones: rho, p log-uniform, Lorentz factor log-uniform in [1, w_hi]
// in an isotropic direction; primitives and conserved, SoA [5][n].
__global__ void seeded_zones_kernel(uint64_t seed, int64_t n, double rho_lo, double rho_hi, double p_lo, double p_hi,
                                    double w_hi, double gm, double* prim, double* cons)
{
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    {
        const uint64_t k = uint64_t(i) * 5;
        const double r0 = uniform01(seed, k), r1 = uniform01(seed, k + 1), r2 = uniform01(seed, k + 2);
        const double r3 = uniform01(seed, k + 3), r4 = uniform01(seed, k + 4);
        const double rho = rho_lo * exp(r0 * log(rho_hi / rho_lo));
        const double pg = p_lo * exp(r1 * log(p_hi / p_lo));
        const double W = exp(r2 * log(w_hi));
        const double ub = sqrt(W * W - 1.0);
        const double mu = 2.0 * r3 - 1.0;
        const double ph = 2.0 * M_PI * r4;
        const double st = sqrt(1.0 - mu * mu);
        const double q[5] = {rho, ub * st * cos(ph), ub * st * sin(ph), ub * mu, pg};
        double u[5];
        conserved_density(q, gm, u);
        for (int c = 0; c < 5; ++c)
        {
            prim[c * n + i] = q[c];
            cons[c * n + i] = u[c];
        }
    }
}

} // namespace srhd
} // namespace mara

using namespace mara;

namespace mara {
namespace srhd {

// One fixed face per thread: the reference's riemann_solver in HLLE or HLLC mode.
__global__ void riemann_kernel(const double* pl, const double* pr, int64_t n, int axis, double gm, int solver,
                               double* f, int32_t* status)
{
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    {
        const double* a = pl + 5 * i;
        const double* b = pr + 5 * i;
        const SPrim<double> L{a[0], {a[1], a[2], a[3]}, a[4]};
        const SPrim<double> R{b[0], {b[1], b[2], b[3]}, b[4]};
        double F[5];
        int bad = 0;
        if (solver == 1) bad = hllc(L, R, axis, gm, F);
        else hlle(L, R, axis, gm, F);
        for (int k = 0; k < 5; ++k) f[5 * i + k] = F[k];
        if (status) status[i] = bad;
    }
}

} // namespace srhd
} // namespace mara

extern "C" {

int mara_srhd_recover_primitive(const double* cons, int64_t n, int64_t component_stride, int64_t zone_stride,
                                double gamma_law_index, double temperature_floor, const void* mlp_weights,
                                int32_t refine32, int32_t seeded_budget, double* prim, int32_t* iterations,
                                int32_t* status, unsigned long long* failures, void* stream)
{
    MARA_REQUIRE(n >= 0, "mara_srhd_recover_primitive: negative zone count");
    if (n == 0) return MARA_OK;
    MARA_REQUIRE(cons && prim, "mara_srhd_recover_primitive: null buffer");
    MARA_REQUIRE(component_stride > 0 && zone_stride > 0, "mara_srhd_recover_primitive: strides must be positive");
    MARA_REQUIRE(gamma_law_index > 1.0, "mara_srhd_recover_primitive: gamma_law_index must exceed 1");
    MARA_REQUIRE(refine32 >= 0 && refine32 <= 16, "mara_srhd_recover_primitive: refine32 must be in [0, 16]");
    const bool seeded = mlp_weights != nullptr || refine32 > 0;
    MARA_REQUIRE(!seeded || (seeded_budget >= 1 && seeded_budget <= 50),
                 "mara_srhd_recover_primitive: seeded_budget must be in [1, 50]");
    srhd::C2PArgs a;
    a.cons = cons;
    a.prim = prim;
    a.n = n;
    a.cs = component_stride;
    a.zs = zone_stride;
    a.gamma = gamma_law_index;
    a.floor = temperature_floor;
    a.iterations = iterations;
    a.status = status;
    a.failures = failures;
    a.mlp = static_cast<const mlp::Weights*>(mlp_weights);
    a.refine32 = refine32;
    a.seeded_budget = seeded_budget;
    cudaStream_t s = as_stream(stream);
    if (mlp_weights == nullptr)
    {
        int blocks = int(std::min<int64_t>((n + 255) / 256, 152 * 16));
        if (refine32 == 0)
            srhd::c2p_default_kernel<<<blocks, srhd::kDefaultThreads, 0, s>>>(a);
        else
            srhd::c2p_refined_kernel<<<blocks, 256, 0, s>>>(a);
        return launch_status("c2p kernel");
    }
    int blocks = int(std::min<int64_t>((n + mlp::kZones - 1) / mlp::kZones, 152 * 8));
    srhd::c2p_mlp_kernel<<<blocks, mlp::kThreads, 0, s>>>(a);
    return launch_status("c2p_mlp_kernel");
}

// ------------------------------------------------------------- host-buffer recovery
// The zones of a host-buffer call go through the GPU in chunks, each on one
// of kHostSlots streams: its copy in, its recovery and its copy out are
// ordered on that stream, and the streams run side by side, so the host-link
// transfers of some chunks overlap the recovery of others. A slot's device
// buffers (conserved and primitives of one chunk, one failure counter) are
// reused by every kHostSlots-th chunk, which the stream order makes safe.
namespace {
constexpr int kHostSlots = 3;

int64_t host_chunk_zones(int64_t n, int32_t chunks) { return (n + chunks - 1) / chunks; }

int64_t host_slot_bytes(int64_t m) { return (10 * m * 8 + 8 + 255) / 256 * 256; }
} // namespace

int64_t mara_srhd_host_workspace_bytes(int64_t n, int32_t chunks)
{
    if (n < 0 || chunks < 1) return -1;
    return kHostSlots * host_slot_bytes(host_chunk_zones(n, chunks)) + 256;
}

int mara_srhd_recover_primitive_host(const double* host_cons, int64_t n, double gamma_law_index,
                                     double temperature_floor, const void* mlp_weights, int32_t refine32,
                                     int32_t seeded_budget, double* host_prim, int32_t chunks, void* workspace,
                                     unsigned long long* failures, void* stream)
{
    MARA_REQUIRE(n >= 0, "mara_srhd_recover_primitive_host: negative zone count");
    MARA_REQUIRE(chunks >= 1 && chunks <= 4096, "mara_srhd_recover_primitive_host: chunks must be in [1, 4096]");
    if (failures) *failures = 0;
    if (n == 0) return MARA_OK;
    MARA_REQUIRE(host_cons && host_prim && workspace, "mara_srhd_recover_primitive_host: null buffer");
    const int64_t m = host_chunk_zones(n, chunks);
    const int64_t slot_bytes = host_slot_bytes(m);
    char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(workspace) + 255) & ~uintptr_t(255));
    cudaStream_t caller = as_stream(stream);
    cudaStream_t st[kHostSlots] = {};
    cudaEvent_t start = nullptr;
    int r = MARA_OK;
    auto cuda = [&](cudaError_t e, const char* what) {
        if (r == MARA_OK && e != cudaSuccess) r = cuda_fail(e, what);
        return r == MARA_OK;
    };
    // the chunks follow whatever the caller queued on its stream before the call
    cuda(cudaEventCreateWithFlags(&start, cudaEventDisableTiming), "cudaEventCreate");
    cuda(cudaEventRecord(start, caller), "cudaEventRecord");
    for (int k = 0; k < kHostSlots && r == MARA_OK; ++k)
    {
        cuda(cudaStreamCreateWithFlags(&st[k], cudaStreamNonBlocking), "cudaStreamCreate");
        cuda(cudaStreamWaitEvent(st[k], start, 0), "cudaStreamWaitEvent");
        auto* count = reinterpret_cast<unsigned long long*>(base + k * slot_bytes + 10 * m * 8);
        cuda(cudaMemsetAsync(count, 0, sizeof(unsigned long long), st[k]), "cudaMemsetAsync");
    }
    for (int64_t c = 0; c * m < n && r == MARA_OK; ++c)
    {
        const int k = int(c % kHostSlots);
        const int64_t z0 = c * m, mz = std::min(m, n - z0);
        auto* dc = reinterpret_cast<double*>(base + k * slot_bytes);
        double* dp = dc + 5 * m;
        auto* count = reinterpret_cast<unsigned long long*>(dc + 10 * m);
        // five component rows of mz zones: from pitch n (host) to pitch m (device)
        if (!cuda(cudaMemcpy2DAsync(dc, m * 8, host_cons + z0, n * 8, mz * 8, 5, cudaMemcpyHostToDevice, st[k]),
                  "cudaMemcpy2DAsync (in)"))
            break;
        const int rr = mara_srhd_recover_primitive(dc, mz, m, 1, gamma_law_index, temperature_floor, mlp_weights,
                                                   refine32, seeded_budget, dp, nullptr, nullptr, count, st[k]);
        if (rr != MARA_OK)
        {
            r = rr;
            break;
        }
        cuda(cudaMemcpy2DAsync(host_prim + z0, n * 8, dp, m * 8, mz * 8, 5, cudaMemcpyDeviceToHost, st[k]),
             "cudaMemcpy2DAsync (out)");
    }
    unsigned long long total = 0;
    for (int k = 0; k < kHostSlots; ++k)
    {
        if (!st[k]) continue;
        if (r == MARA_OK)
        {
            unsigned long long v = 0;
            auto* count = reinterpret_cast<unsigned long long*>(base + k * slot_bytes + 10 * m * 8);
            if (cuda(cudaMemcpyAsync(&v, count, sizeof v, cudaMemcpyDeviceToHost, st[k]), "cudaMemcpyAsync") &&
                cuda(cudaStreamSynchronize(st[k]), "cudaStreamSynchronize"))
                total += v;
        }
        else cudaStreamSynchronize(st[k]);
        cudaStreamDestroy(st[k]);
    }
    if (start) cudaEventDestroy(start);
    if (r == MARA_OK && failures) *failures = total;
    return r;
}

int mara_srhd_seeded_zones(uint64_t seed, int64_t n, double rho_lo, double rho_hi, double p_lo, double p_hi,
                           double w_hi, double gamma_law_index, double* prim, double* cons, void* stream)
{
    MARA_REQUIRE(n >= 0, "mara_srhd_seeded_zones: negative count");
    if (n == 0) return MARA_OK;
    MARA_REQUIRE(prim && cons, "mara_srhd_seeded_zones: null buffer");
    MARA_REQUIRE(rho_lo > 0 && rho_hi >= rho_lo && p_lo > 0 && p_hi >= p_lo && w_hi >= 1.0,
                 "mara_srhd_seeded_zones: bad ranges");
    int blocks = int(std::min<int64_t>((n + 255) / 256, 152 * 16));
    srhd::seeded_zones_kernel<<<blocks, 256, 0, as_stream(stream)>>>(seed, n, rho_lo, rho_hi, p_lo, p_hi, w_hi,
                                                                     gamma_law_index, prim, cons);
    return launch_status("seeded_zones_kernel");
}

int mara_srhd_riemann(const double* pl, const double* pr, int64_t n, int32_t axis, double gamma_law_index,
                      int32_t solver, double* f, int32_t* status, void* stream)
{
    MARA_REQUIRE(n >= 0, "mara_srhd_riemann: negative count");
    MARA_REQUIRE(axis >= 1 && axis <= 3, "mara_srhd_riemann: axis must be 1, 2 or 3");
    MARA_REQUIRE(solver == 0 || solver == 1, "mara_srhd_riemann: solver must be 0 (HLLE) or 1 (HLLC)");
    if (n == 0) return MARA_OK;
    MARA_REQUIRE(pl && pr && f, "mara_srhd_riemann: null buffer");
    int blocks = int(std::min<int64_t>((n + 255) / 256, 152 * 16));
    srhd::riemann_kernel<<<blocks, 256, 0, as_stream(stream)>>>(pl, pr, n, axis - 1, gamma_law_index, solver, f,
                                                                status);
    return launch_status("riemann_kernel");
}

} // extern "C"
