// ORACLE — test infrastructure only.
//
// CPU restatement of the reference's algorithms for the Godunov finite-volume
// update (Mara3p). Only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline leg load or run anything under oracle/; the product path never does.
//
// Shared helpers: the counter-based RNG used by every seeded input generator,
// and a tiny thread pool that runs one task per mesh block per stage, the way
// the reference's compute_threaded executes block tasks on mara::ThreadPool
// (src/parallel_computable.cpp:248-296, src/parallel_thread_pool.hpp:121-199).
#pragma once
#include <atomic>
#include <cstdint>
#include <functional>
#include <thread>
#include <vector>

namespace oracle {

// splitmix64 keyed by (seed, index): the same integer recipe is used on the
// device, so CPU and GPU generate bit-identical seeded inputs.
inline uint64_t hash64(uint64_t seed, uint64_t index)
{
    uint64_t z = seed + (index + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Uniform double in [0, 1) from the top 53 bits of the hash.
inline double uniform01(uint64_t seed, uint64_t index)
{
    return double(hash64(seed, index) >> 11) * 0x1.0p-53;
}

// Run task(k) for k in [0, count) on `threads` workers (threads <= 1: inline).
inline void parallel_for(int count, int threads, const std::function<void(int)>& task)
{
    if (threads <= 1 || count <= 1)
    {
        for (int k = 0; k < count; ++k) task(k);
        return;
    }
    std::atomic<int> next{0};
    std::vector<std::thread> pool;
    for (int w = 0; w < threads; ++w)
    {
        pool.emplace_back([&] {
            for (int k = next++; k < count; k = next++) task(k);
        });
    }
    for (auto& t : pool) t.join();
}

} // namespace oracle
