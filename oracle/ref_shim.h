// ref_shim.h -- TEST INFRASTRUCTURE: host stand-ins for the CUDA built-ins that the
// reference's plain per-node kernels use, so that their unmodified text compiles with
// g++ and runs on the CPU (oracle/build_ref.py).  Nothing here is part of the product.
//
// Execution model: a launch runs its blocks one after another.  Kernels without
// __syncthreads run each block's threads one after another too (ref_launch_seq);
// a kernel with __syncthreads runs the threads of one block as std::threads that
// meet at a std::barrier (ref_launch_sync), with `extern __shared__` storage
// shared by the running block.  Atomics are serialised by one mutex.
#pragma once
#include <algorithm>
#include <barrier>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

using std::isfinite;

struct ref_dim3 {
    unsigned x = 1, y = 1, z = 1;
};
inline thread_local ref_dim3 threadIdx;
inline thread_local ref_dim3 blockIdx;
inline ref_dim3 blockDim;
inline ref_dim3 gridDim;
inline thread_local std::barrier<>* ref_bar = nullptr;
inline std::mutex ref_atomic_mutex;

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __constant__ static
#define __shared__

// storage behind `extern __shared__` arrays (one block runs at a time)
float sdata[4096];

inline void __syncthreads() { ref_bar->arrive_and_wait(); }

inline float atomicAdd(float* p, float v) {
    std::lock_guard<std::mutex> g(ref_atomic_mutex);
    const float o = *p;
    *p = o + v;
    return o;
}
inline int atomicAdd(int* p, int v) {
    std::lock_guard<std::mutex> g(ref_atomic_mutex);
    const int o = *p;
    *p = o + v;
    return o;
}
inline int atomicOr(int* p, int v) {
    std::lock_guard<std::mutex> g(ref_atomic_mutex);
    const int o = *p;
    *p = o | v;
    return o;
}

// grid of `grid` blocks of `block` threads, no block-level synchronisation
inline void ref_launch_seq(unsigned grid, unsigned block, const std::function<void()>& body) {
    blockDim = ref_dim3{block, 1, 1};
    gridDim = ref_dim3{grid, 1, 1};
    for (unsigned b = 0; b < grid; ++b)
        for (unsigned t = 0; t < block; ++t) {
            blockIdx = ref_dim3{b, 0, 0};
            threadIdx = ref_dim3{t, 0, 0};
            body();
        }
}

// the same with the threads of a block running concurrently and meeting at __syncthreads
inline void ref_launch_sync(unsigned grid, unsigned block, const std::function<void()>& body) {
    blockDim = ref_dim3{block, 1, 1};
    gridDim = ref_dim3{grid, 1, 1};
    for (unsigned b = 0; b < grid; ++b) {
        std::barrier<> bar((std::ptrdiff_t)block);
        std::vector<std::thread> th;
        th.reserve(block);
        for (unsigned t = 0; t < block; ++t)
            th.emplace_back([&, b, t] {
                blockIdx = ref_dim3{b, 0, 0};
                threadIdx = ref_dim3{t, 0, 0};
                ref_bar = &bar;
                body();
            });
        for (auto& x : th) x.join();
    }
}
