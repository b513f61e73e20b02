// Shared device helpers for libwcfd: vector loads, block/grid reductions in fp64 and a
// bounded grid barrier for the persistent (cooperatively launched) solver kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "wcfd.h"

namespace wcfd {

constexpr int kBlock = 256;      // threads of the one-thread-per-face/cell kernels
constexpr int kSolverBlock = 512;  // threads of the persistent Krylov kernels
constexpr int kMaxSlots = 6;     // faces per cell (hex)
constexpr int kClusterBlock = 1024;  // threads per CTA of the cluster-resident solver

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ float comp(const float4& v, int o) {
    return o == 0 ? v.x : (o == 1 ? v.y : (o == 2 ? v.z : v.w));
}
__device__ __forceinline__ void set_comp(float4& v, int o, float x) {
    if (o == 0) v.x = x; else if (o == 1) v.y = x; else if (o == 2) v.z = x; else v.w = x;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Longest a block waits at a grid barrier before it gives up and flags
// WCFD_BARRIER_TIMEOUT (a healthy wait is one solver phase: microseconds).
constexpr uint64_t kBarrierTimeoutNs = 1500ull * 1000ull * 1000ull;

// Sum NV doubles over the block; the result is valid in every thread.
template <int NV, int BS>
__device__ __forceinline__ void block_sum(double (&v)[NV]) {
    __shared__ double red[NV][BS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        double x = v[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) red[i][wid] = x;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; ++i) {
        double x = lane < BS / 32 ? red[i][lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        v[i] = x;
    }
    __syncthreads();
}

// Grid-wide synchronisation state living in caller-provided global memory.
//   flags[b]   phase number block b has reached (zeroed before each launch)
//   partials   [2 phase parities][4 values][WCFD_MAX_BLOCKS] per-block partial sums
struct GridCtl {
    double* partials;
    unsigned* flags;
    int* err;
};

// Barrier + reduction over all blocks of a cooperative launch, for phase number `phase`
// (1, 2, 3, ... in every block).  Each block publishes its NV partial sums and then its
// flag with one release store (no atomics); every block waits for all flags (one thread
// per flag, in parallel) and sums the partials in block-index order, so every block gets
// the same bits on every run.  Partials are double-buffered by phase parity: a block can
// only overwrite a buffer after every block has passed the phase that read it.
// Every wait is bounded: on timeout the block sets *err and returns false.
template <int NV, int BS>
__device__ bool grid_sync(const GridCtl& g, double* v, unsigned phase) {
    __shared__ int s_fail;
    if (threadIdx.x == 0) s_fail = 0;
    if constexpr (NV > 0) {
        double t[NV];
#pragma unroll
        for (int i = 0; i < NV; ++i) t[i] = v[i];
        block_sum<NV, BS>(t);
        if (threadIdx.x == 0) {
            double* pb = g.partials + (size_t)(phase & 1u) * 4 * WCFD_MAX_BLOCKS;
#pragma unroll
            for (int i = 0; i < NV; ++i) pb[i * WCFD_MAX_BLOCKS + blockIdx.x] = t[i];
        }
    }
    __syncthreads();  // this block's writes of the phase happen before its release
    if (threadIdx.x == 0) st_release(g.flags + blockIdx.x, phase);
    double acc[NV > 0 ? NV : 1];
#pragma unroll
    for (int i = 0; i < (NV > 0 ? NV : 1); ++i) acc[i] = 0.0;
    bool ok = true;
    for (int j = threadIdx.x; j < (int)gridDim.x; j += BS) {
        if ((int)(ld_acquire(g.flags + j) - phase) < 0) {
            const uint64_t t0 = global_ns();
            unsigned spins = 0;
            while ((int)(ld_acquire(g.flags + j) - phase) < 0) {
                if ((++spins & 31u) == 0u && global_ns() - t0 > kBarrierTimeoutNs) {
                    ok = false;
                    break;
                }
                __nanosleep(20);
            }
        }
        if (!ok) break;
        if constexpr (NV > 0) {
            const double* pb = g.partials + (size_t)(phase & 1u) * 4 * WCFD_MAX_BLOCKS;
#pragma unroll
            for (int i = 0; i < NV; ++i) acc[i] += __ldcg(pb + i * WCFD_MAX_BLOCKS + j);
        }
    }
    if (!ok) {
        atomicExch(g.err, WCFD_BARRIER_TIMEOUT);
        s_fail = 1;
    }
    if constexpr (NV > 0) {
        block_sum<NV, BS>(acc);  // contains __syncthreads, so s_fail is visible after it
#pragma unroll
        for (int i = 0; i < NV; ++i) v[i] = acc[i];
    } else {
        __syncthreads();
    }
    return s_fail == 0;
}

}  // namespace wcfd
