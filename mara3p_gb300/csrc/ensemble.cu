// Batched minidisk ensemble: many independent meshes advanced together.
//
// The reference advances one mesh per process, block by block on a thread
// pool, and folds several steps between host-side reports
// (problems/minidisk.cpp:174-213). Small meshes cannot fill a GB300 that way:
// a 128^2 mesh is 20 warps of sweep work, and every step is three launches.
// Here the members share the GPU:
//
//   MARA_MIXED  every RK stage of all members is ONE persistent launch of the
//               warp-strip sweep over a device work-list. The host lays the
//               28-column strips of all members end to end, cuts their rows
//               into equal chunks and records each chunk's pieces
//               (member, strip, row range). Static mode gives warp w chunk w
//               (one balanced range per warp); dynamic mode cuts finer chunks
//               that warps claim from an atomic counter.
//   MARA_FP64   the tiled FP64 stage kernel per member (no tunables).
//
// Each RK step (both stages plus one clock launch for all members) is a CUDA
// graph captured once and replayed, so a step costs one graph launch on the
// host. The launch shape (resident CTAs per SM, chunks per warp) is chosen by
// timing the candidates on the members themselves.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>
#include "minidisk_device.cuh"

namespace mara {
namespace md {
namespace {

constexpr int kMinItemRows = 4;    // shorter strip tails join the item before them

int strips_of(int n, int cols) { return (n + cols - 1) / cols; }

int64_t plan_work(const int32_t* sizes, int count, int64_t chunks, int cols, std::vector<int4>* items,
                  std::vector<int>* first)
{
    int64_t total = 0;
    for (int m = 0; m < count; ++m) total += int64_t(strips_of(sizes[m], cols)) * sizes[m];
    if (items) items->clear();
    if (first) first->assign(size_t(chunks + 1), 0);
    auto bound = [&](int64_t k) { return total / chunks * k + (total % chunks) * k / chunks; };
    int64_t pos = 0, chunk = 0, n_items = 0;
    for (int m = 0; m < count; ++m)
        for (int sy = 0; sy < strips_of(sizes[m], cols); ++sy)
            for (int i = 0; i < sizes[m];)
            {
                while (bound(chunk + 1) <= pos)
                {
                    ++chunk;
                    if (first) (*first)[size_t(chunk)] = int(n_items);
                }
                int take = int(std::min<int64_t>(sizes[m] - i, bound(chunk + 1) - pos));
                if (sizes[m] - i - take < kMinItemRows) take = sizes[m] - i;
                if (items) items->push_back(make_int4(m, sy, i, i + take));
                ++n_items;
                i += take;
                pos += take;
            }
    while (chunk < chunks)
    {
        ++chunk;
        if (first) (*first)[size_t(chunk)] = int(n_items);
    }
    return n_items;
}

// ------------------------------------------------------------- kernels
__device__ inline int claim_chunk(unsigned* counter, int lane)
{
    unsigned c = 0;
    if (lane == 0) c = atomicAdd(counter, 1u);
    return int(__shfl_sync(0xffffffffu, c, 0));
}

// One stage of every member. counter[0] hands out chunks, counter[1] counts
// finished warps; the last warp to finish returns both to zero for the next
// launch (no warp waits on another).
// MINB: CTAs per SM the register budget is compiled for (1: unconstrained);
// COLS: columns per lane (the 1- or 2-column sweep).
template<int KIND, int MINB, int COLS>
__global__ void __launch_bounds__(SW_WARPS * 32, MINB)
ensemble_sweep_kernel(const Args* __restrict__ table, const int4* __restrict__ items,
                      const int* __restrict__ first, int nchunks, int dynamic, unsigned* counter)
{
    extern __shared__ __align__(16) unsigned char ring_smem[];   // two-column form: RING_WARP_BYTES per warp
    const int lane = threadIdx.x & 31;
    const int warp = blockIdx.x * SW_WARPS + (threadIdx.x >> 5);
    const int warps = gridDim.x * SW_WARPS;
    unsigned char* ring_base = ring_smem + (threadIdx.x >> 5) * RING_WARP_BYTES;
    const Ring2 ring{reinterpret_cast<double2*>(ring_base), reinterpret_cast<float2*>(ring_base + RING_U_BYTES)};
    int chunk = dynamic ? claim_chunk(counter, lane) : warp;
    while (chunk < nchunks)
    {
        const int end = __ldg(first + chunk + 1);
        for (int it = __ldg(first + chunk); it < end; ++it)
        {
            const int4 w = __ldg(items + it);
            const Args A = table[w.x];
            if constexpr (COLS == 2) sweep_strip2<KIND, false, true>(A, w.z, w.w, w.y, ring);
            else sweep_strip<KIND>(A, w.z, w.w, w.y);
        }
        chunk = dynamic ? claim_chunk(counter, lane) : chunk + warps;
    }
    if (dynamic && lane == 0)
    {
        __threadfence();
        if (atomicAdd(counter + 1, 1u) == unsigned(warps - 1))
        {
            atomicExch(counter, 0u);
            atomicExch(counter + 1, 0u);
        }
    }
}

// Two lanes per member (an aligned pair of one warp): the member's two stage
// binaries (FP64 Kepler solves) run side by side.
__global__ void ensemble_clock_kernel(mara_minidisk_clock* clocks, const ClockArgs* args, int count,
                                      int end_step, int begin_step, int key_state)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int m = t >> 1;
    if (m >= count) return;   // both lanes of the pair
    ClockArgs a = args[m];
    a.end_step = end_step;
    a.begin_step = begin_step;
    a.key_state = key_state;
    advance_clock(clocks + m, a, t & 1, 2);
}

struct CopyJob
{
    const double* src;
    double* dst;
    long long n;
};

__global__ void ensemble_copy_kernel(const CopyJob* jobs)
{
    const CopyJob j = jobs[blockIdx.y];
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < j.n; k += stride) j.dst[k] = j.src[k];
}

int device_sms(int* sms, int* dev)
{
    MARA_CUDA(cudaGetDevice(dev));
    MARA_CUDA(cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, *dev));
    return MARA_OK;
}

// Register-budget variants of the sweep kernels: 0 unconstrained, 1 and 2
// compiled for more resident CTAs per SM (5 and 6 for the 1-column sweep, 3
// and 4 for the 2-column one), at the cost of a few bytes of per-item spills.
constexpr int kRegVariants = 3;

template<int KIND, int COLS, int V>
constexpr auto sweep_variant()
{
    constexpr int minb = V == 0 ? 1 : (COLS == 1 ? (V == 1 ? 5 : 6) : (V == 1 ? 3 : 4));
    return ensemble_sweep_kernel<KIND, minb, COLS>;
}

template<int KIND, int COLS>
auto sweep_variant(int v)
{
    return v == 0 ? sweep_variant<KIND, COLS, 0>() : (v == 1 ? sweep_variant<KIND, COLS, 1>() : sweep_variant<KIND, COLS, 2>());
}

template<int KIND>
auto sweep_function(int cols, int v)
{
    return cols == 2 ? sweep_variant<KIND, 2>(v) : sweep_variant<KIND, 1>(v);
}

// shared memory of the two-column sweep's row rings (one per warp)
inline size_t ring_bytes(int cols) { return cols == 2 ? size_t(SW_WARPS) * RING_WARP_BYTES : 0; }

template<int KIND>
int launch_sweep_variant(int cols, int variant, int blocks, cudaStream_t s, const Args* table, const int4* items,
                         const int* first, int nchunks, int dynamic, unsigned* counter)
{
    sweep_function<KIND>(cols, variant)<<<blocks, SW_WARPS * 32, ring_bytes(cols), s>>>(table, items, first, nchunks,
                                                                                      dynamic, counter);
    return launch_status("ensemble sweep kernel");
}

template<int KIND>
int sweep_occupancy(int cols, int variant, int* blocks)
{
    MARA_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, sweep_function<KIND>(cols, variant), SW_WARPS * 32,
                                                             ring_bytes(cols)));
    if (*blocks < 1) *blocks = 1;
    return MARA_OK;
}

// Tuned launch shapes by (device, precision, rk order, sorted mesh sizes).
std::mutex g_tuned_mutex;
std::map<std::string, mara_ensemble_config> g_tuned;

} // namespace
} // namespace md
} // namespace mara

using namespace mara;
using namespace mara::md;

struct mara_minidisk_ensemble
{
    int device = 0, sms = 0, count = 0, rk_order = 2, precision = MARA_MIXED, dt_mode = MARA_DT_CFL;
    int flips = 1;                       // the final state of a step lands in the other buffer
    int occupancy[2][3] = {{1, 1, 1}, {1, 1, 1}};   // resident sweep CTAs per SM: [columns - 1][register variant]
    bool even = true;                    // every member's N is even (the 2-column sweep can run)
    std::vector<mara_minidisk_params> params;
    std::vector<int32_t> sizes;
    std::vector<double*> states, alt;
    std::vector<float*> d1;
    mara_minidisk_clock* clocks = nullptr;
    // host copies of the stage arguments: [slot][member], slots 0-3 = (phase, stage),
    // 4-5 = tuning copies of phase 0 without the wavespeed reduction
    std::vector<Args> host_table;
    Args* table = nullptr;               // device copy of host_table
    ClockArgs* clock_args = nullptr;
    CopyJob* copy_jobs = nullptr;
    unsigned* counters = nullptr;        // [stage][2]
    void* scratch = nullptr;             // alternate states and increments
    int4* items = nullptr;
    int* first = nullptr;
    int64_t nchunks = 0;
    int grid_blocks = 0;
    mara_ensemble_config config{};
    cudaStream_t capture = nullptr;
    cudaGraphExec_t g_begin = nullptr, g_step[2] = {nullptr, nullptr}, g_last[2] = {nullptr, nullptr};
};

namespace {

constexpr int kSlots = 6;

int release_graphs(mara_minidisk_ensemble* e)
{
    cudaGraphExec_t* all[] = {&e->g_begin, &e->g_step[0], &e->g_step[1], &e->g_last[0], &e->g_last[1]};
    for (cudaGraphExec_t* g : all)
        if (*g)
        {
            cudaGraphExecDestroy(*g);
            *g = nullptr;
        }
    return MARA_OK;
}

void release(mara_minidisk_ensemble* e)
{
    if (!e) return;
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(e->device);
    release_graphs(e);
    void* bufs[] = {e->table, e->clock_args, e->copy_jobs, e->counters, e->scratch, e->items, e->first};
    for (void* b : bufs)
        if (b) cudaFree(b);
    if (e->capture) cudaStreamDestroy(e->capture);
    cudaSetDevice(cur);
    delete e;
}

// Enqueue both stages of one step at buffer phase `phase` (0: the members'
// own states hold the step's input). tuning: phase-0 copies that skip the
// wavespeed reduction, so that timing runs change nothing but scratch.
int enqueue_stages(mara_minidisk_ensemble* e, int phase, bool tuning, cudaStream_t s)
{
    const int stages = e->rk_order;
    for (int st = 0; st < stages; ++st)
    {
        const int slot = tuning ? 4 + st : phase * 2 + st;
        if (e->precision == MARA_MIXED)
        {
            const Args* t = e->table + size_t(slot) * e->count;
            const int dyn = e->config.chunks_per_warp > 1;
            unsigned* c = e->counters + 2 * st;
            const int v = e->config.register_variant, cols = e->config.cols_per_lane;
            int r = st == 1 ? launch_sweep_variant<K_MIX2>(cols, v, e->grid_blocks, s, t, e->items, e->first,
                                                           int(e->nchunks), dyn, c)
                  : stages == 2 ? launch_sweep_variant<K_MIXD>(cols, v, e->grid_blocks, s, t, e->items, e->first,
                                                               int(e->nchunks), dyn, c)
                                : launch_sweep_variant<K_MIX1>(cols, v, e->grid_blocks, s, t, e->items, e->first,
                                                               int(e->nchunks), dyn, c);
            if (r) return r;
        }
        else
        {
            for (int m = 0; m < e->count; ++m)
                if (int r = grid_stage(e->host_table[size_t(slot) * e->count + m], K_FP64, s)) return r;
        }
    }
    return MARA_OK;
}

// phase: the buffer phase of the step that just ran; the mixed CFL
// conversion reads the step's result, the other buffer when steps flip
int enqueue_clock(mara_minidisk_ensemble* e, int end_step, int begin_step, int phase, cudaStream_t s)
{
    const int key_state = e->flips ? 1 - phase : 0;
    ensemble_clock_kernel<<<(2 * e->count + 31) / 32, 32, 0, s>>>(e->clocks, e->clock_args, e->count, end_step,
                                                                  begin_step, key_state);
    return launch_status("ensemble clock kernel");
}

int enqueue_copy_back(mara_minidisk_ensemble* e, cudaStream_t s)
{
    ensemble_copy_kernel<<<dim3(std::max(1, 2 * e->sms / std::max(1, e->count / 8 + 1)), e->count), 256, 0, s>>>(e->copy_jobs);
    return launch_status("ensemble copy kernel");
}

template<typename F>
int capture_graph(mara_minidisk_ensemble* e, cudaGraphExec_t* out, F&& body)
{
    MARA_CUDA(cudaStreamBeginCapture(e->capture, cudaStreamCaptureModeRelaxed));
    int r = body(e->capture);
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(e->capture, &g);
    if (r == MARA_OK && ce != cudaSuccess) r = cuda_fail(ce, "cudaStreamEndCapture");
    if (r == MARA_OK)
    {
        cudaError_t ie = cudaGraphInstantiate(out, g, 0);
        if (ie != cudaSuccess) r = cuda_fail(ie, "cudaGraphInstantiate");
        // uploaded now, so that the first replay costs what the later ones do
        else if ((ie = cudaGraphUpload(*out, e->capture)) != cudaSuccess) r = cuda_fail(ie, "cudaGraphUpload");
    }
    if (g) cudaGraphDestroy(g);
    return r;
}

int build_graphs(mara_minidisk_ensemble* e)
{
    release_graphs(e);
    if (int r = capture_graph(e, &e->g_begin, [&](cudaStream_t s) { return enqueue_clock(e, 0, 1, 0, s); })) return r;
    for (int p = 0; p < (e->flips ? 2 : 1); ++p)
    {
        if (int r = capture_graph(e, &e->g_step[p], [&](cudaStream_t s) {
                if (int q = enqueue_stages(e, p, false, s)) return q;
                return enqueue_clock(e, 1, 1, p, s);
            })) return r;
        if (int r = capture_graph(e, &e->g_last[p], [&](cudaStream_t s) {
                if (int q = enqueue_stages(e, p, false, s)) return q;
                if (int q = enqueue_clock(e, 1, 0, p, s)) return q;
                return e->flips && p == 0 ? enqueue_copy_back(e, s) : MARA_OK;
            })) return r;
    }
    return MARA_OK;
}

int check_config(const mara_minidisk_ensemble* e, const mara_ensemble_config& c)
{
    MARA_REQUIRE(c.register_variant >= 0 && c.register_variant < kRegVariants,
                 "minidisk ensemble: register_variant must be 0, 1 or 2");
    MARA_REQUIRE(c.cols_per_lane == 1 || c.cols_per_lane == 2, "minidisk ensemble: cols_per_lane must be 1 or 2");
    MARA_REQUIRE(c.cols_per_lane == 1 || e->precision != MARA_MIXED || e->even,
                 "minidisk ensemble: cols_per_lane 2 needs every member's mesh size to be even");
    const int occ = e->occupancy[c.cols_per_lane - 1][c.register_variant];
    MARA_REQUIRE(c.blocks_per_sm >= 1 && c.blocks_per_sm <= occ,
                 "minidisk ensemble: blocks_per_sm must be in [1, " + std::to_string(occ) + "]");
    MARA_REQUIRE(c.chunks_per_warp >= 1 && c.chunks_per_warp <= 64, "minidisk ensemble: chunks_per_warp must be in [1, 64]");
    return MARA_OK;
}

// Make `c` the launch shape: plan its work-list, upload it, size the
// persistent grid. On failure nothing of the ensemble changes. The graphs
// still name the previous work-list until build_graphs runs.
int apply_config(mara_minidisk_ensemble* e, const mara_ensemble_config& c)
{
    if (int r = check_config(e, c)) return r;
    if (e->precision != MARA_MIXED)
    {
        e->config = c;
        return MARA_OK;
    }
    const int grid_blocks = c.blocks_per_sm * e->sms;
    const int64_t nchunks = int64_t(grid_blocks) * SW_WARPS * c.chunks_per_warp;
    std::vector<int4> items;
    std::vector<int> first;
    plan_work(e->sizes.data(), e->count, nchunks, c.cols_per_lane == 2 ? SW2_COLS : SW_COLS, &items, &first);
    int4* d_items = nullptr;
    int* d_first = nullptr;
    auto undo = [&](cudaError_t err, const char* what) {
        if (d_items) cudaFree(d_items);
        if (d_first) cudaFree(d_first);
        return cuda_fail(err, what);
    };
    cudaError_t err;
    if ((err = cudaMalloc(&d_items, items.size() * sizeof(int4))) != cudaSuccess) return undo(err, "cudaMalloc(items)");
    if ((err = cudaMalloc(&d_first, first.size() * sizeof(int))) != cudaSuccess) return undo(err, "cudaMalloc(first)");
    if ((err = cudaMemcpy(d_items, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice)) != cudaSuccess)
        return undo(err, "cudaMemcpy(items)");
    if ((err = cudaMemcpy(d_first, first.data(), first.size() * sizeof(int), cudaMemcpyHostToDevice)) != cudaSuccess)
        return undo(err, "cudaMemcpy(first)");
    if (e->items) cudaFree(e->items);
    if (e->first) cudaFree(e->first);
    e->items = d_items;
    e->first = d_first;
    e->grid_blocks = grid_blocks;
    e->nchunks = nchunks;
    e->config = c;
    return MARA_OK;
}

std::string tuning_key(const mara_minidisk_ensemble* e)
{
    std::vector<int32_t> s = e->sizes;
    std::sort(s.begin(), s.end());
    std::string k = std::to_string(e->device) + "/" + std::to_string(e->sms) + "/" + std::to_string(e->precision) + "/" +
                    std::to_string(e->rk_order) + ":";
    for (int32_t n : s) k += std::to_string(n) + ",";
    return k;
}

// Time both stages of one phase-0 step (tuning tables) under e->config: one
// warm-up, then the median of three, in milliseconds.
int time_config(mara_minidisk_ensemble* e, double* ms)
{
    cudaStream_t s = e->capture;
    ScopedEvents events;
    MARA_CUDA(events.create(2));
    cudaEvent_t a = events[0], b = events[1];
    int r = enqueue_stages(e, 0, true, s);
    float t[3] = {0, 0, 0};
    for (int k = 0; r == MARA_OK && k < 3; ++k)
    {
        cudaEventRecord(a, s);
        r = enqueue_stages(e, 0, true, s);
        cudaEventRecord(b, s);
        if (r == MARA_OK)
        {
            cudaError_t ce = cudaEventSynchronize(b);
            if (ce != cudaSuccess) r = cuda_fail(ce, "cudaEventSynchronize");
            else cudaEventElapsedTime(&t[k], a, b);
        }
    }
    std::sort(t, t + 3);
    *ms = t[1];
    return r;
}

int tune(mara_minidisk_ensemble* e)
{
    if (e->precision != MARA_MIXED) return build_graphs(e);
    MARA_CUDA(cudaDeviceSynchronize());
    const mara_ensemble_config keep = e->config;
    mara_ensemble_config best = keep;
    double best_ms = 1e300;
    int r = MARA_OK;
    const int chunk_choices[] = {1, 2, 4, 8};
    for (int cols = 1; r == MARA_OK && cols <= (e->even ? 2 : 1); ++cols)
    for (int v = 0; r == MARA_OK && v < kRegVariants; ++v)
        for (int b = e->occupancy[cols - 1][v]; r == MARA_OK && b >= std::max(1, e->occupancy[cols - 1][v] - 1); --b)
            for (int c : chunk_choices)
            {
                const mara_ensemble_config cand{b, c, cols, v, 0.0};
                double ms = 0;
                if ((r = apply_config(e, cand)) || (r = time_config(e, &ms))) break;
                if (ms < best_ms)
                {
                    best_ms = ms;
                    best = cand;
                    best.stage_ms = ms;
                }
            }
    if (r)
    {
        apply_config(e, keep);
        build_graphs(e);
        return r;
    }
    if (int q = apply_config(e, best)) return q;
    {
        std::lock_guard<std::mutex> lock(g_tuned_mutex);
        g_tuned[tuning_key(e)] = best;
    }
    return build_graphs(e);
}

} // namespace

extern "C" {

int64_t mara_minidisk_ensemble_plan(const int32_t* sizes, int32_t count, int64_t chunks, int32_t strip_columns,
                                    int32_t* items, int64_t capacity, int32_t* chunk_first)
{
    if (!sizes || count < 1 || chunks < 1 || chunks > (int64_t(1) << 30) || capacity < 0 ||
        (strip_columns != SW_COLS && strip_columns != SW2_COLS))
    {
        fail(MARA_ERR_ARGUMENT, "mara_minidisk_ensemble_plan: bad arguments");
        return -1;
    }
    for (int m = 0; m < count; ++m)
        if (sizes[m] < 1 || sizes[m] > 65536)
        {
            fail(MARA_ERR_ARGUMENT, "mara_minidisk_ensemble_plan: mesh size out of range");
            return -1;
        }
    std::vector<int4> it;
    std::vector<int> first;
    const int64_t n = plan_work(sizes, count, chunks, strip_columns, &it, &first);
    if (items)
        for (int64_t k = 0; k < std::min(n, capacity); ++k)
        {
            items[4 * k + 0] = it[size_t(k)].x;
            items[4 * k + 1] = it[size_t(k)].y;
            items[4 * k + 2] = it[size_t(k)].z;
            items[4 * k + 3] = it[size_t(k)].w;
        }
    if (chunk_first) std::copy(first.begin(), first.end(), chunk_first);
    return n;
}

int mara_minidisk_ensemble_create(const mara_minidisk_params* params, int32_t count, double* const* states,
                                  mara_minidisk_clock* clocks, int32_t rk_order, int32_t precision,
                                  int32_t dt_mode, int32_t autotune, mara_minidisk_ensemble** out)
{
    MARA_REQUIRE(out != nullptr, "mara_minidisk_ensemble_create: out is null");
    *out = nullptr;
    MARA_REQUIRE(params && states && clocks, "mara_minidisk_ensemble_create: null argument");
    MARA_REQUIRE(count >= 1 && count <= 65535, "mara_minidisk_ensemble_create: count must be in [1, 65535]");
    MARA_REQUIRE(rk_order == 1 || rk_order == 2, "mara_minidisk_ensemble_create: rk_order must be 1 or 2");
    MARA_REQUIRE(precision == MARA_FP64 || precision == MARA_MIXED, "mara_minidisk_ensemble_create: bad precision");
    MARA_REQUIRE(dt_mode == MARA_DT_FORMULA || dt_mode == MARA_DT_CFL, "mara_minidisk_ensemble_create: bad dt_mode");
    MARA_REQUIRE(autotune >= 0 && autotune <= 2, "mara_minidisk_ensemble_create: autotune must be 0, 1 or 2");
    for (int m = 0; m < count; ++m)
    {
        if (int r = check_params(params + m)) return r;
        const int N = params[m].block_size << params[m].depth;
        MARA_REQUIRE(states[m] != nullptr && (reinterpret_cast<uintptr_t>(states[m]) & 15) == 0,
                     "mara_minidisk_ensemble_create: state " + std::to_string(m) + " is null or not 16-byte aligned");
        MARA_REQUIRE(precision == MARA_FP64 || N >= 64,
                     "mara_minidisk_ensemble_create: MARA_MIXED needs meshes of at least 64^2 (member " +
                     std::to_string(m) + ")");
    }

    auto* e = new mara_minidisk_ensemble;
    auto fail_out = [&](int r) { release(e); return r; };
    e->count = count;
    e->rk_order = rk_order;
    e->precision = precision;
    e->dt_mode = dt_mode;
    e->flips = !(precision == MARA_FP64 && rk_order == 2);
    e->clocks = clocks;
    e->params.assign(params, params + count);
    e->states.assign(states, states + count);
    for (int m = 0; m < count; ++m) e->sizes.push_back(params[m].block_size << params[m].depth);
    if (int r = device_sms(&e->sms, &e->device)) return fail_out(r);
    for (int cols = 1; cols <= 2; ++cols)
        for (int v = 0; v < kRegVariants; ++v)
        {
            int o1 = 1, o2 = 1;
            if (rk_order == 2)
            {
                if (int r = sweep_occupancy<K_MIXD>(cols, v, &o1)) return fail_out(r);
                if (int r = sweep_occupancy<K_MIX2>(cols, v, &o2)) return fail_out(r);
            }
            else
            {
                if (int r = sweep_occupancy<K_MIX1>(cols, v, &o1)) return fail_out(r);
                o2 = o1;
            }
            e->occupancy[cols - 1][v] = std::min(o1, o2);
        }
    for (int m = 0; m < count; ++m) e->even = e->even && e->sizes[m] % 2 == 0;

    // scratch: per member one FP64 state (+ FP32 increment for mixed RK2), 256-byte aligned
    std::vector<size_t> off_alt(count), off_d1(count);
    size_t bytes = 0;
    for (int m = 0; m < count; ++m)
    {
        const size_t NN = size_t(e->sizes[m]) * e->sizes[m];
        off_alt[m] = bytes;
        bytes += (3 * NN * sizeof(double) + 255) / 256 * 256;
        off_d1[m] = bytes;
        if (precision == MARA_MIXED && rk_order == 2) bytes += (3 * NN * sizeof(float) + 255) / 256 * 256;
    }
    if (cudaMalloc(&e->scratch, std::max<size_t>(bytes, 256)) != cudaSuccess)
        return fail_out(fail(MARA_ERR_CUDA, "mara_minidisk_ensemble_create: cannot allocate " + std::to_string(bytes) +
                                            " bytes of scratch"));
    for (int m = 0; m < count; ++m)
    {
        e->alt.push_back(reinterpret_cast<double*>(static_cast<char*>(e->scratch) + off_alt[m]));
        e->d1.push_back(precision == MARA_MIXED && rk_order == 2
                        ? reinterpret_cast<float*>(static_cast<char*>(e->scratch) + off_d1[m]) : nullptr);
    }

    // stage arguments
    e->host_table.resize(size_t(kSlots) * count);
    std::vector<ClockArgs> cargs(count);
    std::vector<CopyJob> jobs(count);
    for (int m = 0; m < count; ++m)
    {
        Args base = base_args(params + m);
        base.clock = clocks + m;
        auto* amax = reinterpret_cast<unsigned long long*>(&clocks[m].max_wavespeed);
        unsigned long long* reduce = dt_mode == MARA_DT_CFL ? amax : nullptr;
        double* buf[2] = {e->states[m], e->alt[m]};
        for (int p = 0; p < 2; ++p)
        {
            Args a1 = base, a2 = base;
            a1.stage = 0;
            a2.stage = 1;
            if (precision == MARA_FP64 && rk_order == 2)
            {
                a1.u_in = buf[0]; a1.u_out = buf[1];
                a2.u_in = buf[1]; a2.u_avg = buf[0]; a2.u_out = buf[0]; a2.amax = reduce;
            }
            else if (rk_order == 2)
            {
                a1.u_in = buf[p]; a1.d_out = e->d1[m];
                a2.u_in = buf[p]; a2.d1 = e->d1[m]; a2.u_out = buf[1 - p]; a2.amax = reduce;
                a2.amax_key = 1;
            }
            else
            {
                a1.u_in = buf[p]; a1.u_out = buf[1 - p]; a1.amax = reduce;
                a1.amax_key = precision == MARA_MIXED;
            }
            e->host_table[size_t(p * 2 + 0) * count + m] = a1;
            e->host_table[size_t(p * 2 + 1) * count + m] = a2;
            if (p == 0)
            {
                a1.amax = nullptr;
                a2.amax = nullptr;
                e->host_table[size_t(4) * count + m] = a1;
                e->host_table[size_t(5) * count + m] = a2;
            }
        }
        cargs[m] = clock_args(params + m, dt_mode, rk_order, 1, 1);
        if (precision == MARA_MIXED && dt_mode == MARA_DT_CFL)
        {
            cargs[m].wavespeed_key = 1;
            cargs[m].u_key[0] = buf[0];
            cargs[m].u_key[1] = buf[1];
        }
        jobs[m] = CopyJob{e->alt[m], e->states[m], (long long)(3 * size_t(e->sizes[m]) * e->sizes[m])};
    }
    auto upload = [&](void** dst, const void* src, size_t n) -> int {
        MARA_CUDA(cudaMalloc(dst, n));
        MARA_CUDA(cudaMemcpy(*dst, src, n, cudaMemcpyHostToDevice));
        return MARA_OK;
    };
    if (int r = upload(reinterpret_cast<void**>(&e->table), e->host_table.data(), e->host_table.size() * sizeof(Args)))
        return fail_out(r);
    if (int r = upload(reinterpret_cast<void**>(&e->clock_args), cargs.data(), cargs.size() * sizeof(ClockArgs)))
        return fail_out(r);
    if (int r = upload(reinterpret_cast<void**>(&e->copy_jobs), jobs.data(), jobs.size() * sizeof(CopyJob)))
        return fail_out(r);
    {
        const unsigned zero[4] = {0, 0, 0, 0};
        if (int r = upload(reinterpret_cast<void**>(&e->counters), zero, sizeof zero)) return fail_out(r);
    }
    if (cudaStreamCreateWithFlags(&e->capture, cudaStreamNonBlocking) != cudaSuccess)
        return fail_out(fail(MARA_ERR_CUDA, "mara_minidisk_ensemble_create: cannot create the capture stream"));

    // launch shape: default, cached, or tuned now
    e->config = e->even && precision == MARA_MIXED ? mara_ensemble_config{e->occupancy[1][0], 1, 2, 0, 0.0}
                                                   : mara_ensemble_config{e->occupancy[0][0], 1, 1, 0, 0.0};
    e->grid_blocks = 0;
    bool tuned = false;
    if (autotune == 1)
    {
        std::lock_guard<std::mutex> lock(g_tuned_mutex);
        auto it = g_tuned.find(tuning_key(e));
        if (it != g_tuned.end())
        {
            e->config = it->second;
            tuned = true;
        }
    }
    int r = MARA_OK;
    if (autotune == 0 || tuned)
    {
        r = apply_config(e, e->config);
        if (r == MARA_OK) r = build_graphs(e);
    }
    else
    {
        r = tune(e);
    }
    if (r) return fail_out(r);
    *out = e;
    return MARA_OK;
}

int mara_minidisk_ensemble_clock_init(mara_minidisk_ensemble* e, double time, void* stream)
{
    MARA_REQUIRE(e != nullptr, "mara_minidisk_ensemble_clock_init: ensemble is null");
    for (int m = 0; m < e->count; ++m)
        if (int r = clock_init(&e->params[m], e->states[m], time, e->clocks + m, e->precision, as_stream(stream)))
            return r;
    return MARA_OK;
}

int mara_minidisk_ensemble_advance(mara_minidisk_ensemble* e, int32_t steps, void* stream)
{
    MARA_REQUIRE(e != nullptr, "mara_minidisk_ensemble_advance: ensemble is null");
    MARA_REQUIRE(steps >= 0, "mara_minidisk_ensemble_advance: negative step count");
    if (steps == 0) return MARA_OK;
    MARA_REQUIRE(e->g_begin && e->g_step[0] && e->g_last[0] && (!e->flips || (e->g_step[1] && e->g_last[1])),
                 "mara_minidisk_ensemble_advance: the step graphs are missing (an earlier reconfiguration failed)");
    cudaStream_t s = as_stream(stream);
    MARA_CUDA(cudaGraphLaunch(e->g_begin, s));
    int phase = 0;
    for (int k = 0; k + 1 < steps; ++k)
    {
        MARA_CUDA(cudaGraphLaunch(e->g_step[phase], s));
        if (e->flips) phase ^= 1;
    }
    MARA_CUDA(cudaGraphLaunch(e->g_last[phase], s));
    return MARA_OK;
}

int mara_minidisk_ensemble_get_config(const mara_minidisk_ensemble* e, mara_ensemble_config* out)
{
    MARA_REQUIRE(e && out, "mara_minidisk_ensemble_get_config: null argument");
    *out = e->config;
    return MARA_OK;
}

int mara_minidisk_ensemble_set_config(mara_minidisk_ensemble* e, const mara_ensemble_config* config)
{
    MARA_REQUIRE(e && config, "mara_minidisk_ensemble_set_config: null argument");
    mara_ensemble_config c = *config;
    c.stage_ms = 0.0;
    if (int r = check_config(e, c)) return r;
    MARA_CUDA(cudaDeviceSynchronize());
    if (int r = apply_config(e, c)) return r;
    return build_graphs(e);
}

int mara_minidisk_ensemble_tune(mara_minidisk_ensemble* e)
{
    MARA_REQUIRE(e != nullptr, "mara_minidisk_ensemble_tune: ensemble is null");
    return tune(e);
}

int mara_minidisk_ensemble_stage_times(mara_minidisk_ensemble* e, int32_t reps, double* ms)
{
    MARA_REQUIRE(e && ms, "mara_minidisk_ensemble_stage_times: null argument");
    MARA_REQUIRE(reps >= 1 && reps <= 1000, "mara_minidisk_ensemble_stage_times: reps must be in [1, 1000]");
    MARA_REQUIRE(e->precision == MARA_MIXED, "mara_minidisk_ensemble_stage_times: MARA_MIXED ensembles only");
    MARA_CUDA(cudaDeviceSynchronize());
    cudaStream_t s = e->capture;
    ScopedEvents ev;   // one per stage boundary: rk_order + 1 <= 3
    MARA_CUDA(ev.create(e->rk_order + 1));
    std::vector<std::vector<float>> t(size_t(e->rk_order));
    int r = enqueue_stages(e, 0, true, s);
    for (int k = 0; r == MARA_OK && k < reps; ++k)
    {
        for (int st = 0; r == MARA_OK && st < e->rk_order; ++st)
        {
            const int slot = 4 + st;
            cudaEventRecord(ev[st], s);
            const Args* tab = e->table + size_t(slot) * e->count;
            const int dyn = e->config.chunks_per_warp > 1;
            unsigned* c = e->counters + 2 * st;
            const int v = e->config.register_variant;
            const int cols = e->config.cols_per_lane;
            r = st == 1 ? launch_sweep_variant<K_MIX2>(cols, v, e->grid_blocks, s, tab, e->items, e->first,
                                                       int(e->nchunks), dyn, c)
              : e->rk_order == 2 ? launch_sweep_variant<K_MIXD>(cols, v, e->grid_blocks, s, tab, e->items, e->first,
                                                                int(e->nchunks), dyn, c)
                                 : launch_sweep_variant<K_MIX1>(cols, v, e->grid_blocks, s, tab, e->items, e->first,
                                                                int(e->nchunks), dyn, c);
        }
        cudaEventRecord(ev[e->rk_order], s);
        if (r == MARA_OK)
        {
            cudaError_t ce = cudaEventSynchronize(ev[e->rk_order]);
            if (ce != cudaSuccess) r = cuda_fail(ce, "cudaEventSynchronize");
            for (int st = 0; r == MARA_OK && st < e->rk_order; ++st)
            {
                float x = 0;
                cudaEventElapsedTime(&x, ev[st], ev[st + 1]);
                t[size_t(st)].push_back(x);
            }
        }
    }
    if (r) return r;
    for (int st = 0; st < e->rk_order; ++st)
    {
        std::vector<float>& v = t[size_t(st)];
        std::sort(v.begin(), v.end());
        ms[st] = v[v.size() / 2];
    }
    return MARA_OK;
}

int mara_minidisk_ensemble_destroy(mara_minidisk_ensemble* e)
{
    if (!e) return MARA_OK;
    cudaError_t err = cudaDeviceSynchronize();
    release(e);
    return err == cudaSuccess ? MARA_OK : cuda_fail(err, "mara_minidisk_ensemble_destroy");
}

} // extern "C"
