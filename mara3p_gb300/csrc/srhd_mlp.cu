// Training of the SRHD pressure-guess MLP (srhd_mlp.cuh) on the GPU with
// hand-written kernels: FP32 forward, backward and Adam.
//
// Training pairs are (conserved, primitive) zones whose primitives come from
// the library's own FP64 recovery (mara_srhd_recover_primitive); the target
// is y = log(p E / q) (srhd_mlp.cuh). Loss: mean squared error of y.
//
// Trainable parameters are the contiguous float run w1, b1, w2, b2, w3, b3 of
// mlp::Weights. Gradients of a batch are accumulated per CTA (128 zones) in
// shared memory and added to a global gradient buffer with atomics.
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <algorithm>
#include "common.cuh"
#include "srhd_mlp.cuh"

namespace mara {
namespace mlp {

constexpr int kParamBegin = offsetof(Weights, w1) / sizeof(float);
constexpr int kParamEnd = (offsetof(Weights, b3) / sizeof(float)) + 1;
constexpr int kParams = kParamEnd - kParamBegin;       // 4545
static_assert(offsetof(Weights, w1) % sizeof(float) == 0, "float layout");
static_assert(offsetof(Weights, out_shift) == offsetof(Weights, b3) + sizeof(float), "contiguous parameters");

constexpr int kTile = 128;       // zones per CTA tile in training

struct TrainSmem
{
    float w1[kHidden][kIn], b1[kHidden], w2[kHidden][kHidden], b2[kHidden], w3[kHidden];
    float h1[kTile][kHidden + 1];
    float da2[kTile][kHidden + 1];
    float x[kTile][kIn];
    float g_w1[kHidden][kIn], g_b1[kHidden], g_b2[kHidden], g_w3[kHidden];
    float g_b3;
    float loss;
};

__device__ inline float* params(Weights* w) { return reinterpret_cast<float*>(w) + kParamBegin; }

// Features and target of the training zones: cons/prim SoA [5][n].
__global__ void prepare_kernel(const double* cons, const double* prim, int64_t n, float* feat, float* target)
{
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    {
        double D = cons[i], S1 = cons[n + i], S2 = cons[2 * n + i], S3 = cons[3 * n + i], tau = cons[4 * n + i];
        float f[4];
        raw_features(D, S1, S2, S3, tau, f);
        for (int k = 0; k < 4; ++k) feat[4 * i + k] = f[k];
        double E, q, SS;
        zone_invariants(D, S1, S2, S3, tau, E, q, SS);
        target[i] = q > 0.0 ? float(log(prim[4 * n + i] * E / q)) : 0.0f;
    }
}

// Column sums and sums of squares of (feat[4], target) for normalisation.
__global__ void moments_kernel(const float* feat, const float* target, int64_t n, double* acc /*10*/)
{
    double s[5] = {0, 0, 0, 0, 0}, q[5] = {0, 0, 0, 0, 0};
    for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    {
        for (int k = 0; k < 4; ++k)
        {
            double v = feat[4 * i + k];
            s[k] += v;
            q[k] += v * v;
        }
        double v = target[i];
        s[4] += v;
        q[4] += v * v;
    }
    for (int k = 0; k < 5; ++k)
    {
        for (int o = 16; o > 0; o >>= 1)
        {
            s[k] += __shfl_xor_sync(0xffffffffu, s[k], o);
            q[k] += __shfl_xor_sync(0xffffffffu, q[k], o);
        }
    }
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 5; ++k)
        {
            atomicAdd(acc + k, s[k]);
            atomicAdd(acc + 5 + k, q[k]);
        }
}

__device__ inline float uniform_pm1(uint64_t seed, uint64_t i)
{
    uint64_t z = seed + (i + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return float(double(z >> 11) * 0x1.0p-53) * 2.f - 1.f;
}

// Normalisation from the moments, Glorot-uniform weights, zero biases.
__global__ void init_kernel(Weights* w, const double* acc, int64_t n, uint64_t seed)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kIn)
    {
        double mean = acc[i] / double(n);
        double var = fmax(acc[5 + i] / double(n) - mean * mean, 1e-12);
        w->norm_shift[i] = float(mean);
        w->norm_scale[i] = float(1.0 / sqrt(var));
    }
    if (i == 0)
    {
        double mean = acc[4] / double(n);
        double var = fmax(acc[9] / double(n) - mean * mean, 1e-12);
        w->out_shift = float(mean);
        w->out_scale = float(sqrt(var));
        w->b3 = 0.f;
    }
    float* p = params(w);
    for (int k = i; k < kParams; k += gridDim.x * blockDim.x)
    {
        int off = kParamBegin + k;
        float v = 0.f;
        if (off < int(offsetof(Weights, b1) / 4))
            v = uniform_pm1(seed, k) * sqrtf(6.f / float(kIn + kHidden));
        else if (off >= int(offsetof(Weights, w2) / 4) && off < int(offsetof(Weights, b2) / 4))
            v = uniform_pm1(seed, k) * sqrtf(6.f / float(kHidden + kHidden));
        else if (off >= int(offsetof(Weights, w3) / 4) && off < int(offsetof(Weights, b3) / 4))
            v = uniform_pm1(seed, k) * sqrtf(6.f / float(kHidden + 1));
        p[k] = v;
    }
}

// Forward + backward over zones idx[begin, begin + count) (idx may be null:
// identity). Adds dLoss/dparam into grad (kParams floats) and the loss sum
// into *loss; loss = sum (out - target)^2 / count.
__global__ void __launch_bounds__(kTile) grad_kernel(const Weights* w, const float* feat, const float* target,
                                                     const int64_t* idx, int64_t begin, int64_t count,
                                                     float* grad, float* loss)
{
    extern __shared__ __align__(16) unsigned char raw[];
    TrainSmem& s = *reinterpret_cast<TrainSmem*>(raw);
    const int tid = threadIdx.x;
    for (int i = tid; i < kHidden * kIn; i += blockDim.x) (&s.w1[0][0])[i] = (&w->w1[0][0])[i];
    for (int i = tid; i < kHidden * kHidden; i += blockDim.x) (&s.w2[0][0])[i] = (&w->w2[0][0])[i];
    for (int i = tid; i < kHidden; i += blockDim.x)
    {
        s.b1[i] = w->b1[i];
        s.b2[i] = w->b2[i];
        s.w3[i] = w->w3[i];
        s.g_b1[i] = 0.f;
        s.g_b2[i] = 0.f;
        s.g_w3[i] = 0.f;
    }
    for (int i = tid; i < kHidden * kIn; i += blockDim.x) (&s.g_w1[0][0])[i] = 0.f;
    if (tid == 0)
    {
        s.g_b3 = 0.f;
        s.loss = 0.f;
    }
    const float b3 = w->b3, out_shift = w->out_shift, out_scale = w->out_scale;
    float shift[4], scale[4];
    for (int k = 0; k < 4; ++k)
    {
        shift[k] = w->norm_shift[k];
        scale[k] = w->norm_scale[k];
    }
    const float inv_count = 1.f / float(count);
    // per-thread accumulators of the W2 gradient: entries tid, tid + 128, ...
    float gw2[kHidden * kHidden / kTile];
    for (int q = 0; q < kHidden * kHidden / kTile; ++q) gw2[q] = 0.f;
    __syncthreads();

    for (int64_t tile = int64_t(blockIdx.x) * kTile; tile < count; tile += int64_t(gridDim.x) * kTile)
    {
        const int64_t r = tile + tid;
        const bool valid = r < count;
        float x[4] = {0, 0, 0, 0};
        float tgt = 0.f;
        if (valid)
        {
            int64_t z = idx ? idx[begin + r] : begin + r;
            for (int k = 0; k < 4; ++k) x[k] = (feat[4 * z + k] - shift[k]) * scale[k];
            tgt = target[z];
        }
        for (int k = 0; k < 4; ++k) s.x[tid][k] = x[k];
        // forward
        for (int j = 0; j < kHidden; ++j)
        {
            float a = s.b1[j] + s.w1[j][0] * x[0] + s.w1[j][1] * x[1] + s.w1[j][2] * x[2] + s.w1[j][3] * x[3];
            s.h1[tid][j] = tanhf(a);
        }
        float y = b3;
        float h2[kHidden];
        for (int n = 0; n < kHidden; ++n)
        {
            float a = s.b2[n];
            for (int k = 0; k < kHidden; ++k) a += s.w2[n][k] * s.h1[tid][k];
            h2[n] = tanhf(a);
            y += s.w3[n] * h2[n];
        }
        float out = out_shift + out_scale * y;
        float err = valid ? out - tgt : 0.f;
        float dy = valid ? 2.f * err * inv_count * out_scale : 0.f;
        // backward through layers 3 and 2
        atomicAdd(&s.loss, err * err * inv_count);
        atomicAdd(&s.g_b3, dy);
        for (int n = 0; n < kHidden; ++n)
        {
            atomicAdd(&s.g_w3[n], dy * h2[n]);
            float da = dy * s.w3[n] * (1.f - h2[n] * h2[n]);
            s.da2[tid][n] = da;
            atomicAdd(&s.g_b2[n], da);
        }
        // back to layer 1
        for (int k = 0; k < kHidden; ++k)
        {
            float dh = 0.f;
            for (int n = 0; n < kHidden; ++n) dh += s.w2[n][k] * s.da2[tid][n];
            float h = s.h1[tid][k];
            float da1 = dh * (1.f - h * h);
            atomicAdd(&s.g_b1[k], da1);
            for (int i = 0; i < kIn; ++i) atomicAdd(&s.g_w1[k][i], da1 * x[i]);
        }
        __syncthreads();
        // W2 gradient: sum over the tile's zones of da2[z][n] * h1[z][k]
        for (int q = 0; q < kHidden * kHidden / kTile; ++q)
        {
            int e = tid + q * kTile;
            int n = e / kHidden, k = e % kHidden;
            float acc = 0.f;
            for (int z = 0; z < kTile; ++z) acc += s.da2[z][n] * s.h1[z][k];
            gw2[q] += acc;
        }
        __syncthreads();
    }
    float* g = grad;
    const int o_w1 = 0, o_b1 = kHidden * kIn, o_w2 = o_b1 + kHidden, o_b2 = o_w2 + kHidden * kHidden;
    const int o_w3 = o_b2 + kHidden, o_b3 = o_w3 + kHidden;
    for (int q = 0; q < kHidden * kHidden / kTile; ++q) atomicAdd(g + o_w2 + tid + q * kTile, gw2[q]);
    for (int i = tid; i < kHidden * kIn; i += blockDim.x) atomicAdd(g + o_w1 + i, (&s.g_w1[0][0])[i]);
    for (int i = tid; i < kHidden; i += blockDim.x)
    {
        atomicAdd(g + o_b1 + i, s.g_b1[i]);
        atomicAdd(g + o_b2 + i, s.g_b2[i]);
        atomicAdd(g + o_w3 + i, s.g_w3[i]);
    }
    if (tid == 0)
    {
        atomicAdd(g + o_b3, s.g_b3);
        atomicAdd(loss, s.loss);
    }
}

__global__ void adam_kernel(Weights* w, const float* grad, float* m, float* v, float lr, float beta1, float beta2,
                            float eps, int step)
{
    float* p = params(w);
    const float c1 = 1.f - powf(beta1, float(step)), c2 = 1.f - powf(beta2, float(step));
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < kParams; k += gridDim.x * blockDim.x)
    {
        float gk = grad[k];
        float mk = beta1 * m[k] + (1.f - beta1) * gk;
        float vk = beta2 * v[k] + (1.f - beta2) * gk * gk;
        m[k] = mk;
        v[k] = vk;
        p[k] -= lr * (mk / c1) / (sqrtf(vk / c2) + eps);
    }
}

__global__ void export_bf16_kernel(Weights* w)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kHidden * kHidden; i += gridDim.x * blockDim.x)
        w->w2_bf16[i / kHidden][i % kHidden] = __float2bfloat16_rn(w->w2[i / kHidden][i % kHidden]);
}

// Evaluate the inference network (BF16 tensor cores) on raw feature rows,
// writing y for each zone: used by tests to compare with the FP32 oracle.
__global__ void __launch_bounds__(kThreads) infer_kernel(const Weights* w, const float* feat, int64_t n, float* y)
{
    __shared__ Shared sm;
    begin(*w, sm);
    uint32_t phase = 0;
    for (int64_t base = int64_t(blockIdx.x) * kZones; base < n; base += int64_t(gridDim.x) * kZones)
    {
        __syncthreads();
        for (int t = threadIdx.x; t < kZones; t += blockDim.x)
        {
            float f[4] = {0, 0, 0, 0};
            if (base + t < n)
                for (int k = 0; k < 4; ++k) f[k] = feat[4 * (base + t) + k];
            stage_features(sm, t, f);
        }
        __syncthreads();
        forward(sm, phase);
        __syncthreads();
        for (int t = threadIdx.x; t < kZones; t += blockDim.x)
            if (base + t < n) y[base + t] = sm.out[t];
    }
    end(sm);
}

int grad_launch(const Weights* w, const float* feat, const float* target, const int64_t* idx, int64_t begin,
                int64_t count, float* grad, float* loss, cudaStream_t s)
{
    static PerDeviceOnce once;
    int dev = 0;
    MARA_CUDA(cudaGetDevice(&dev));
    if (int r = once.run(dev, []() -> int {
            MARA_CUDA(cudaFuncSetAttribute(grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           int(sizeof(TrainSmem))));
            return MARA_OK;
        }))
        return r;
    int blocks = int(std::min<int64_t>((count + kTile - 1) / kTile, 152 * 2));
    grad_kernel<<<blocks, kTile, sizeof(TrainSmem), s>>>(w, feat, target, idx, begin, count, grad, loss);
    return launch_status("grad_kernel");
}

} // namespace mlp
} // namespace mara

using namespace mara;
using namespace mara::mlp;

extern "C" {

int64_t mara_srhd_mlp_weights_bytes(void) { return int64_t(sizeof(Weights)); }

int32_t mara_srhd_mlp_param_count(void) { return kParams; }

// Workspace layout, every region 256-byte aligned: features float[n][4],
// targets float[n], gradient / Adam m / Adam v float[kParams] each, loss
// float, moments double[10].
struct Layout
{
    int64_t feat, target, grad, m, v, loss, moments, total;
};

static int64_t align256(int64_t x) { return (x + 255) & ~int64_t(255); }

static Layout layout(int64_t n)
{
    Layout L;
    L.feat = 0;
    L.target = align256(L.feat + n * 4 * int64_t(sizeof(float)));
    L.grad = align256(L.target + n * int64_t(sizeof(float)));
    L.m = align256(L.grad + kParams * int64_t(sizeof(float)));
    L.v = align256(L.m + kParams * int64_t(sizeof(float)));
    L.loss = align256(L.v + kParams * int64_t(sizeof(float)));
    L.moments = align256(L.loss + int64_t(sizeof(float)));
    L.total = align256(L.moments + 10 * int64_t(sizeof(double)));
    return L;
}

int64_t mara_srhd_mlp_workspace_bytes(int64_t n) { return n > 0 ? layout(n).total : -1; }

int mara_srhd_mlp_prepare(const double* cons, const double* prim, int64_t n, void* weights, uint64_t seed,
                          void* workspace, void* stream)
{
    MARA_REQUIRE(n > 0 && cons && prim && weights && workspace, "mara_srhd_mlp_prepare: bad argument");
    cudaStream_t s = as_stream(stream);
    char* ws = static_cast<char*>(workspace);
    const Layout L = layout(n);
    float* feat = reinterpret_cast<float*>(ws + L.feat);
    float* target = reinterpret_cast<float*>(ws + L.target);
    double* acc = reinterpret_cast<double*>(ws + L.moments);
    MARA_CUDA(cudaMemsetAsync(acc, 0, 10 * sizeof(double), s));
    int blocks = int(std::min<int64_t>((n + 255) / 256, 152 * 8));
    prepare_kernel<<<blocks, 256, 0, s>>>(cons, prim, n, feat, target);
    if (int r = launch_status("prepare_kernel")) return r;
    moments_kernel<<<blocks, 256, 0, s>>>(feat, target, n, acc);
    if (int r = launch_status("moments_kernel")) return r;
    MARA_CUDA(cudaMemsetAsync(weights, 0, sizeof(Weights), s));
    init_kernel<<<(kParams + 255) / 256, 256, 0, s>>>(static_cast<Weights*>(weights), acc, n, seed);
    if (int r = launch_status("init_kernel")) return r;
    export_bf16_kernel<<<16, 256, 0, s>>>(static_cast<Weights*>(weights));
    return launch_status("export_bf16_kernel");
}

int mara_srhd_mlp_gradient(const void* weights, const void* workspace, int64_t n, float* grad, float* loss,
                           void* stream)
{
    MARA_REQUIRE(n > 0 && weights && workspace && grad && loss, "mara_srhd_mlp_gradient: bad argument");
    cudaStream_t s = as_stream(stream);
    const char* ws = static_cast<const char*>(workspace);
    const Layout L = layout(n);
    const float* feat = reinterpret_cast<const float*>(ws + L.feat);
    const float* target = reinterpret_cast<const float*>(ws + L.target);
    MARA_CUDA(cudaMemsetAsync(grad, 0, kParams * sizeof(float), s));
    MARA_CUDA(cudaMemsetAsync(loss, 0, sizeof(float), s));
    return grad_launch(static_cast<const Weights*>(weights), feat, target, nullptr, 0, n, grad, loss, s);
}

int mara_srhd_mlp_train(void* weights, void* workspace, int64_t n, const int64_t* order, int32_t steps,
                        int32_t batch, float lr, float* loss_history, void* stream)
{
    MARA_REQUIRE(n > 0 && weights && workspace && order, "mara_srhd_mlp_train: bad argument");
    MARA_REQUIRE(steps >= 0 && batch > 0 && batch <= n, "mara_srhd_mlp_train: bad steps or batch");
    cudaStream_t s = as_stream(stream);
    char* ws = static_cast<char*>(workspace);
    const Layout L = layout(n);
    const float* feat = reinterpret_cast<const float*>(ws + L.feat);
    const float* target = reinterpret_cast<const float*>(ws + L.target);
    float* grad = reinterpret_cast<float*>(ws + L.grad);
    float* m = reinterpret_cast<float*>(ws + L.m);
    float* v = reinterpret_cast<float*>(ws + L.v);
    float* loss = reinterpret_cast<float*>(ws + L.loss);
    MARA_CUDA(cudaMemsetAsync(m, 0, kParams * sizeof(float), s));
    MARA_CUDA(cudaMemsetAsync(v, 0, kParams * sizeof(float), s));
    Weights* w = static_cast<Weights*>(weights);
    int64_t cursor = 0;
    for (int step = 1; step <= steps; ++step)
    {
        if (cursor + batch > n) cursor = 0;
        MARA_CUDA(cudaMemsetAsync(grad, 0, kParams * sizeof(float), s));
        MARA_CUDA(cudaMemsetAsync(loss, 0, sizeof(float), s));
        if (int r = grad_launch(w, feat, target, order, cursor, batch, grad, loss, s)) return r;
        cursor += batch;
        adam_kernel<<<(kParams + 255) / 256, 256, 0, s>>>(w, grad, m, v, lr, 0.9f, 0.999f, 1e-8f, step);
        if (int r = launch_status("adam_kernel")) return r;
        if (loss_history)
            MARA_CUDA(cudaMemcpyAsync(loss_history + (step - 1), loss, sizeof(float), cudaMemcpyDeviceToDevice, s));
    }
    export_bf16_kernel<<<16, 256, 0, s>>>(w);
    return launch_status("export_bf16_kernel");
}

int mara_srhd_mlp_infer(const void* weights, const float* features, int64_t n, float* y, void* stream)
{
    MARA_REQUIRE(n >= 0, "mara_srhd_mlp_infer: negative count");
    if (n == 0) return MARA_OK;
    MARA_REQUIRE(weights && features && y, "mara_srhd_mlp_infer: null buffer");
    int blocks = int(std::min<int64_t>((n + kZones - 1) / kZones, 152 * 8));
    infer_kernel<<<blocks, kThreads, 0, as_stream(stream)>>>(static_cast<const Weights*>(weights), features, n, y);
    return launch_status("infer_kernel");
}

} // extern "C"
