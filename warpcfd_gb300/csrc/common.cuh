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
struct GridCtl {
    double* partials;   // [8][WCFD_MAX_BLOCKS]
    double* results;    // [8]
    unsigned* bar;      // [0] arrival count, [1] generation
    int* err;           // status word shared by all blocks of the launch
};

// Barrier over all blocks of a cooperative launch.  When NV > 0 the last block to
// arrive sums the NV per-block partials (v[] of every block) in block-index order, so
// every run and every block gets the same bits, and publishes them in results[] before
// releasing the others; on return v[] holds the grid-wide sums.  Every wait is bounded:
// on timeout the block sets *err and returns false, as it does when another block has
// already flagged an error.
template <int NV, int BS>
__device__ bool grid_sync(const GridCtl& g, double* v) {
    __shared__ int s_last, s_fail;
    __shared__ unsigned s_gen;
    if constexpr (NV > 0) {
        double t[NV];
#pragma unroll
        for (int i = 0; i < NV; ++i) t[i] = v[i];
        block_sum<NV, BS>(t);
        if (threadIdx.x == 0) {
#pragma unroll
            for (int i = 0; i < NV; ++i) g.partials[i * WCFD_MAX_BLOCKS + blockIdx.x] = t[i];
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        s_fail = 0;
        const unsigned gen = ld_acquire(g.bar + 1);
        s_gen = gen;
        __threadfence();
        const unsigned prev = atomicAdd(g.bar, 1u);
        s_last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (s_last) {
        __threadfence();
        if constexpr (NV > 0) {
            double acc[NV];
#pragma unroll
            for (int i = 0; i < NV; ++i) {
                double a = 0.0;
                for (int b = threadIdx.x; b < (int)gridDim.x; b += BS)
                    a += __ldcg(g.partials + i * WCFD_MAX_BLOCKS + b);
                acc[i] = a;
            }
            block_sum<NV, BS>(acc);
            if (threadIdx.x == 0) {
#pragma unroll
                for (int i = 0; i < NV; ++i) g.results[i] = acc[i];
            }
            __threadfence();
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            atomicExch(g.bar, 0u);
            __threadfence();
            st_release(g.bar + 1, s_gen + 1u);
        }
    } else if (threadIdx.x == 0) {
        const uint64_t t0 = global_ns();
        unsigned spins = 0;
        while (ld_acquire(g.bar + 1) == s_gen) {
            if ((++spins & 63u) == 0u && global_ns() - t0 > kBarrierTimeoutNs) {
                atomicExch(g.err, WCFD_BARRIER_TIMEOUT);
                s_fail = 1;
                break;
            }
            __nanosleep(32);
        }
    }
    __syncthreads();
    __threadfence();
    if (threadIdx.x == 0 && !s_fail) {
        if (*((volatile int*)g.err) != 0) s_fail = 1;
    }
    __syncthreads();
    if (s_fail) return false;
    if constexpr (NV > 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) v[i] = __ldcg(g.results + i);
    }
    return true;
}

}  // namespace wcfd
