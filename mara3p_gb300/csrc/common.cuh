// Shared helpers of the mara_gb300 library: error reporting for the C ABI and
// the FP64 binary orbit (used on the host and on the device).
#pragma once
#include <cuda_runtime.h>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <mutex>
#include <string>
#include "mara_gb300.h"

namespace mara {

// Record `msg` as the calling thread's last error and return `code`.
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

#define MARA_CUDA(call)                                                     \
    do {                                                                    \
        cudaError_t e_ = (call);                                            \
        if (e_ != cudaSuccess) return ::mara::cuda_fail(e_, #call);         \
    } while (0)

#define MARA_REQUIRE(cond, msg)                                             \
    do {                                                                    \
        if (!(cond)) return ::mara::fail(MARA_ERR_ARGUMENT, (msg));         \
    } while (0)

inline int launch_status(const char* what)
{
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? MARA_OK : cuda_fail(e, what);
}

inline cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

// One-time set-up per device (a kernel attribute, an occupancy query) that is
// safe to reach from several host threads. Only a set-up that succeeded is
// remembered: one that failed returns its status to its caller and runs again
// on the next call. Devices are indexed modulo 64.
struct PerDeviceOnce
{
    std::atomic<bool> done[64] = {};
    std::mutex m;

    template<typename F>
    int run(int dev, F&& setup)
    {
        std::atomic<bool>& d = done[dev & 63];
        if (d.load(std::memory_order_acquire)) return MARA_OK;
        std::lock_guard<std::mutex> lock(m);
        if (d.load(std::memory_order_relaxed)) return MARA_OK;
        const int r = setup();
        if (r == MARA_OK) d.store(true, std::memory_order_release);
        return r;
    }
};

// Timing events owned by a scope: every event created is destroyed when the
// holder goes, so an early return on a failed call leaks none.
struct ScopedEvents
{
    cudaEvent_t ev[8] = {};
    int n = 0;
    ScopedEvents() = default;
    ScopedEvents(const ScopedEvents&) = delete;
    ScopedEvents& operator=(const ScopedEvents&) = delete;
    ~ScopedEvents()
    {
        for (int k = 0; k < n; ++k) cudaEventDestroy(ev[k]);
    }
    // count (at most 8) events with default flags
    cudaError_t create(int count)
    {
        for (; n < count && n < 8; ++n)
            if (cudaError_t e = cudaEventCreate(&ev[n])) return e;
        return count <= 8 ? cudaSuccess : cudaErrorInvalidValue;
    }
    cudaEvent_t operator[](int k) const { return ev[k]; }
};

// Binary state in the rotating frame at time t: the Kepler orbit of
// src/physics_two_body.hpp:54-157 (a = 1, M = 1, G = 1) rotated by -omega_frame*t
// (rotate/transform, :395-444), in the reference's evaluation order. The
// Newton solve for the eccentric anomaly is capped at 200 iterations so that
// it always terminates on the device.
struct Binary { double m1, x1, y1, vx1, vy1, m2, x2, y2, vx2, vy2; };

__host__ __device__ inline Binary binary_state(double q, double e, double omega_frame, double t)
{
    const double G = 1.0, a = 1.0, M = 1.0;
    const double W = sqrt(G * M / a / a / a);
    const double Mt = W * t;
    double E = Mt;
    for (int it = 0; it < 200; ++it)
    {
        double f = E - e * sin(E) - Mt;
        if (!(fabs(f) > 1e-12)) break;
        E -= f / (1 - e * cos(E));
    }
    const double mu = q / (1.0 + q);
    const double M1 = M * (1.0 - mu);
    const double M2 = M * mu;
    const double x1  = -a * mu * (e - cos(E));
    const double y1  = +a * mu * (0 + sin(E)) * sqrt(1 - e * e);
    const double x2  = -x1 / q;
    const double y2  = -y1 / q;
    const double vx1 = -a * mu * W / (1 - e * cos(E)) * sin(E);
    const double vy1 = +a * mu * W / (1 - e * cos(E)) * cos(E) * sqrt(1 - e * e);
    const double vx2 = -vx1 / q;
    const double vy2 = -vy1 / q;
    const double angle = -omega_frame * t;
    const double c = cos(-angle);
    const double s = sin(-angle);
    Binary b;
    b.m1 = M1;
    b.x1 = +x1 * c + y1 * s + 0.0;
    b.y1 = -x1 * s + y1 * c + 0.0;
    b.vx1 = +vx1 * c + vy1 * s + 0.0;
    b.vy1 = -vx1 * s + vy1 * c + 0.0;
    b.m2 = M2;
    b.x2 = +x2 * c + y2 * s + 0.0;
    b.y2 = -x2 * s + y2 * c + 0.0;
    b.vx2 = +vx2 * c + vy2 * s + 0.0;
    b.vy2 = -vx2 * s + vy2 * c + 0.0;
    return b;
}

} // namespace mara
