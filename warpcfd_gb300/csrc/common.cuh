// Shared device helpers for libwcfd: vector loads, block/grid reductions in fp64 and a
// bounded grid barrier for the persistent (cooperatively launched) solver kernels.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>
#include <climits>

#include "wcfd.h"

namespace wcfd {

constexpr int kBlock = 256;      // threads of the one-thread-per-face/cell kernels
constexpr int kMaxFieldBlock = 512;  // largest block of the batched field kernels (a launch parameter)
constexpr int kSolverBlock = 1024;  // threads of the persistent Krylov kernels (one block per SM)
constexpr int kMaxSlots = 6;     // faces per cell (hex)
// face reference of a null slot: a cell of a mixed mesh with fewer faces than the
// mesh's faces_per_cell (a wedge or a tetrahedron among hexes); its weights are zero
constexpr int kNullSlot = INT_MIN;
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

// ---------------------------------------------------------------------------------
// fp64-accurate dot products without per-element fp64 arithmetic.
//
// GB300 executes fp64 at about 1/64 of its fp32 rate, so a cast and an fp64 FMA per
// element would dominate a bandwidth-bound Krylov phase.  Instead each product is formed
// exactly as an unevaluated sum h + r (TwoProduct with an FMA) and accumulated in
// float-float arithmetic (Knuth's TwoSum), the "Dot2" scheme of Ogita, Rump and Oishi,
// "Accurate sum and dot product", SIAM J. Sci. Comput. 26 (2005): the result is as accurate
// as if it were computed in twice the working precision.  Totals are merged in float-float
// across warps, blocks and CTAs in a fixed order (TwoSum merges are exact up to the low
// word) and converted to fp64 once, by one thread: a full-warp fp64 instruction is itself
// expensive on GB300.
// __fmul_rn / __fadd_rn keep the compiler from contracting the error-free transforms.
struct ff {
    float hi, lo;
};

__device__ __forceinline__ ff ff_zero() { return ff{0.0f, 0.0f}; }

// acc += a * b
__device__ __forceinline__ void ff_fma(ff& acc, float a, float b) {
    const float h = __fmul_rn(a, b);
    const float r = fmaf(a, b, -h);
    const float s = __fadd_rn(acc.hi, h);
    const float bb = __fsub_rn(s, acc.hi);
    const float q = __fadd_rn(__fsub_rn(acc.hi, __fsub_rn(s, bb)), __fsub_rn(h, bb));
    acc.hi = s;
    acc.lo = __fadd_rn(acc.lo, __fadd_rn(q, r));
}

// a += b (symmetric: merging a into b gives the same bits, so butterfly shuffles agree)
__device__ __forceinline__ void ff_merge(ff& a, const ff& b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    const float q = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
    a.hi = s;
    a.lo = __fadd_rn(__fadd_rn(a.lo, b.lo), q);
}

__device__ __forceinline__ void ff_shfl_merge(ff& v, int o) {
    ff t;
    t.hi = __shfl_xor_sync(0xffffffffu, v.hi, o);
    t.lo = __shfl_xor_sync(0xffffffffu, v.lo, o);
    ff_merge(v, t);
}

__device__ __forceinline__ double ff_to_double(const ff& v) { return (double)v.hi + (double)v.lo; }

// Scalar float-float arithmetic for the Krylov recurrences.  One dependent fp64 operation
// costs about 64 cycles on GB300 and an fp64 division about 600, against about 5 and 50
// for fp32, and the thread that forms alpha and beta holds up every other thread of the
// solve; so alpha = rz / pq, beta = rz' / rz and the stop test are evaluated on the
// float-float sums directly.

// (hi, lo) with |lo| <= ulp(hi) / 2 (Dekker's fast two-sum; the sums above keep |lo| small)
__device__ __forceinline__ ff ff_norm(const ff& a) {
    const float s = __fadd_rn(a.hi, a.lo);
    return ff{s, __fsub_rn(a.lo, __fsub_rn(s, a.hi))};
}
__device__ __forceinline__ ff ff_from_double(double d) {
    const float h = (float)d;
    return ff{h, (float)(d - (double)h)};
}
// a > b and a <= b for normalised operands (both false when either is NaN, as for fp64)
__device__ __forceinline__ bool ff_gt(const ff& a, const ff& b) {
    return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo);
}
__device__ __forceinline__ bool ff_le(const ff& a, const ff& b) {
    return a.hi < b.hi || (a.hi == b.hi && a.lo <= b.lo);
}
// a + b of two floats as a normalised float-float (TwoSum)
__device__ __forceinline__ ff ff_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return ff{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
// a * b in float-float (TwoProduct of the high words plus the cross terms)
__device__ __forceinline__ ff ff_mul(const ff& a, const ff& b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
    return ff_norm(ff{p, e});
}
// a / b in float-float (see ff_div_to_float); b.hi != 0
__device__ __forceinline__ ff ff_div(const ff& an, const ff& bn) {
    const ff a = ff_norm(an), b = ff_norm(bn);
    const float q1 = __fdiv_rn(a.hi, b.hi);
    const float p = __fmul_rn(q1, b.hi);
    const float e = fmaf(q1, b.hi, -p);
    const float rh = __fsub_rn(a.hi, p);
    const float rl = __fsub_rn(__fsub_rn(a.lo, e), __fmul_rn(q1, b.lo));
    const float q2 = __fdiv_rn(__fadd_rn(rh, rl), b.hi);
    return ff_two_sum(q1, q2);
}
__device__ __forceinline__ float ff_to_float(const ff& a) { return __fadd_rn(a.hi, a.lo); }

// a / b rounded to fp32: a float quotient q1, the remainder a - q1 b formed exactly
// (TwoProduct; a.hi - q1 b.hi is exact by Sterbenz's lemma), one correction q2; q1 + q2
// agrees with a / b to about 2^-46 before the final rounding.  b.hi != 0.
__device__ __forceinline__ float ff_div_to_float(const ff& an, const ff& bn) {
    const ff a = ff_norm(an), b = ff_norm(bn);
    const float q1 = __fdiv_rn(a.hi, b.hi);
    const float p = __fmul_rn(q1, b.hi);
    const float e = fmaf(q1, b.hi, -p);
    const float rh = __fsub_rn(a.hi, p);
    const float rl = __fsub_rn(__fsub_rn(a.lo, e), __fmul_rn(q1, b.lo));
    const float q2 = __fdiv_rn(__fadd_rn(rh, rl), b.hi);
    return __fadd_rn(q1, q2);
}

// Block total of NV float-float accumulators, still as float-float (the same bits in every
// thread).  Warps merge by butterfly shuffles, then warp 0 merges the warp totals; no fp64
// instruction is issued (a full-warp fp64 instruction is expensive on GB300).
template <int NV, int BS>
__device__ __forceinline__ void block_reduce_ff(ff (&v)[NV]) {
    __shared__ ff wsum[NV][BS / 32];
    __shared__ ff res[NV];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) ff_shfl_merge(v[i], o);
        if (lane == 0) wsum[i][wid] = v[i];
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            ff x = lane < BS / 32 ? wsum[i][lane] : ff_zero();
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) ff_shfl_merge(x, o);
            if (lane == 0) res[i] = x;
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = res[i];
    __syncthreads();
}

// Grid-wide synchronisation state living in caller-provided global memory.
//   flags[WCFD_MAX_BLOCKS + 2]  arrival counter (zeroed before each launch)
//   partials   [2 phase parities][2 float4 slots][WCFD_MAX_BLOCKS] per-block float-float
//              totals, two values (hi, lo, hi, lo) per float4
struct GridCtl {
    double* partials;
    unsigned* flags;
    int* err;
};

__device__ __forceinline__ void red_release_add(unsigned* p, unsigned v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Barrier + reduction over all blocks of a cooperative launch, for phase number `phase`
// (1, 2, 3, ... in every block).  v[] holds this block's float-float totals (from
// block_reduce_ff); on return out[] holds the grid-wide sums (normalised float-float).
//
// Thread 0 of every block stores the block's totals (two values per float4), then adds
// one to a single arrival counter with a release reduction and waits (acquire loads) for
// the counter to reach phase x gridDim.x.  Then warp 0 of every block reads all blocks'
// totals and merges them in the same fixed order (lane-strided over blocks, then a
// butterfly), so every block holds the same bits on every run without a second hop.
// Measured on GB300 (2,000 barriers of two sums, cooperative launch): 2.47 us per barrier
// at 152 blocks, against 3.4 us for an aggregator barrier (per-block flags, block 0
// merging and releasing a `done` word) and 1.26 us for the counter alone.  The all-read
// cost grows with the number of blocks (4.7 us at 456: every block requests the same
// lines), so the Krylov kernels run one 1,024-thread block per SM.  Totals are double-
// buffered by phase parity: a buffer is rewritten only after every block has passed the
// phase that read it.  The wait is bounded: on timeout the block sets *err and returns
// false.  NV <= 4.
template <int NV, int BS>
__device__ bool grid_sync(const GridCtl& g, const ff* v, ff* out, unsigned phase) {
    static_assert(NV >= 1 && NV <= 4, "grid_sync carries 1..4 sums");
    constexpr int NQ = (NV + 1) / 2;
    __shared__ int s_fail;
    __shared__ ff s_res[NV];
    float4* pb = reinterpret_cast<float4*>(g.partials) + (size_t)(phase & 1u) * NQ * WCFD_MAX_BLOCKS;
    unsigned* ctr = g.flags + WCFD_MAX_BLOCKS + 2;
    if (threadIdx.x == 0) {
        s_fail = 0;
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            const ff a = v[2 * q];
            const ff b = 2 * q + 1 < NV ? v[2 * q + 1] : ff_zero();
            pb[q * WCFD_MAX_BLOCKS + blockIdx.x] = make_float4(a.hi, a.lo, b.hi, b.lo);
        }
    }
    __syncthreads();  // every thread's writes of the phase happen before the release below
    if (threadIdx.x == 0) {
        red_release_add(ctr, 1u);
        const unsigned target = phase * gridDim.x;
        if ((int)(ld_acquire(ctr) - target) < 0) {
            const uint64_t t0 = global_ns();
            unsigned spins = 0;
            while ((int)(ld_acquire(ctr) - target) < 0) {
                if ((++spins & 31u) == 0u && global_ns() - t0 > kBarrierTimeoutNs) {
                    s_fail = 1;
                    atomicExch(g.err, WCFD_BARRIER_TIMEOUT);
                    break;
                }
            }
        }
    }
    __syncthreads();
    if (s_fail) return false;
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        ff x[2 * NQ];
#pragma unroll
        for (int i = 0; i < 2 * NQ; ++i) x[i] = ff_zero();
        for (int k = lane; k < (int)gridDim.x; k += 32) {
#pragma unroll
            for (int q = 0; q < NQ; ++q) {
                const float4 t = __ldcg(pb + q * WCFD_MAX_BLOCKS + k);
                ff_merge(x[2 * q], ff{t.x, t.y});
                ff_merge(x[2 * q + 1], ff{t.z, t.w});
            }
        }
#pragma unroll
        for (int i = 0; i < NV; ++i) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) ff_shfl_merge(x[i], o);
            if (lane == 0) s_res[i] = ff_norm(x[i]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; ++i) out[i] = s_res[i];
    __syncthreads();
    return true;
}

// NVTX range over a host scope (a stage of a step), for Nsight Systems timelines: one
// cheap call each way when no tool is attached (NVTX v3, header-only)
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

}  // namespace wcfd
