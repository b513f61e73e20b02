// Thread-block-cluster primitives shared by the cluster-resident solvers: rank queries,
// the hardware cluster barrier, distributed-shared-memory loads and stores, and a
// deterministic float-float all-reduce over the CTAs of a cluster.
#pragma once

#include "common.cuh"

namespace wcfd {

constexpr int CBS = kClusterBlock;

__device__ __forceinline__ unsigned cluster_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cluster_nranks() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// shared::cluster address of `p` (a pointer into this CTA's shared memory) in CTA `rank`
__device__ __forceinline__ uint32_t map_rank(const void* p, unsigned rank) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}
// Loads stay ordered against the cluster barrier (both are volatile asm) but carry no
// memory clobber, so the compiler may keep several of them in flight.
__device__ __forceinline__ float ld_cluster_f32(uint32_t addr) {
    float v;
    asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(addr));
    return v;
}
// value at packed column cp = (rank << 24) | local of an array laid out like `base` in
// every CTA: a plain shared-memory load when this CTA owns it, a DSMEM load otherwise
__device__ __forceinline__ float ld_col(const float* base, uint32_t cp, unsigned me) {
    const unsigned rk = cp >> 24;
    const uint32_t lo = cp & 0xFFFFFFu;
    if (rk == me) return base[lo];
    return ld_cluster_f32(map_rank(base + lo, rk));
}
__device__ __forceinline__ void st_cluster_v2f32(uint32_t addr, float a, float b) {
    asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" :: "r"(addr), "f"(a), "f"(b) : "memory");
}

// All-reduce over the cluster of NV float-float accumulators: the CTA total is stored
// into slot `me` of every CTA's shared memory, and after the barrier warp 0 of each CTA
// merges the cs slots in a fixed order and one thread converts to fp64, so every CTA gets
// the same bits.  Slots are double-buffered by `parity`.
template <int NV>
__device__ __forceinline__ void cluster_allreduce(ff (&acc)[NV], double (&out)[NV], ff* slots, unsigned parity,
                                                  unsigned me, unsigned cs) {
    __shared__ double res[NV];
    block_reduce_ff<NV, CBS>(acc);
    ff* base = slots + parity * (NV * 16);
    if (threadIdx.x < cs) {
#pragma unroll
        for (int i = 0; i < NV; ++i)
            st_cluster_v2f32(map_rank(base + i * 16 + me, threadIdx.x), acc[i].hi, acc[i].lo);
    }
    cluster_sync_all();
    if (threadIdx.x < 32) {
        const unsigned lane = threadIdx.x;
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            ff x = lane < cs ? base[i * 16 + lane] : ff_zero();
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) ff_shfl_merge(x, o);
            if (lane == 0) res[i] = ff_to_double(x);
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < NV; ++i) out[i] = res[i];
}

// Sum NV float-float accumulators over the CTAs of the cluster.  The result (fp64) is left
// in thread 0 of every CTA only (the same bits in every CTA); the caller derives its
// scalars there and broadcasts them with one __syncthreads.  Costs one __syncthreads and
// one cluster barrier: warps merge by butterfly shuffles, warp 0 merges the warp totals
// and stores the CTA total into slot `me` of every CTA (DSMEM), and after the barrier
// warp 0 merges the cs slots in rank order.  wsum [2][NV][32] and slots [2][NV][16] are
// double-buffered by `parity`.
template <int NV>
__device__ __forceinline__ void cluster_reduce_to_thread0(ff (&acc)[NV], double (&out)[NV], ff* wsum, ff* slots,
                                                          unsigned parity, unsigned me, unsigned cs) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) ff_shfl_merge(acc[i], o);
        if (lane == 0) wsum[(parity * NV + i) * 32 + wid] = acc[i];
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            ff x = lane < CBS / 32 ? wsum[(parity * NV + i) * 32 + lane] : ff_zero();
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) ff_shfl_merge(x, o);
            if ((unsigned)lane < cs) st_cluster_v2f32(map_rank(slots + (parity * NV + i) * 16 + me, lane), x.hi, x.lo);
        }
    }
    cluster_sync_all();
    if (wid == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            ff y = (unsigned)lane < cs ? slots[(parity * NV + i) * 16 + lane] : ff_zero();
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) ff_shfl_merge(y, o);
            if (lane == 0) out[i] = ff_to_double(y);
        }
    }
}

// Sum NV float-float values over the CTAs of the cluster, result (float-float, the same bits
// in every CTA) in thread 0 only.  The block stage is a shared-memory tree instead of a
// butterfly in every warp, so that most warps issue one store and wait: every thread
// stores its values into sbuf [NV][CBS]; threads 0..255 merge four each (t, t+256, t+512,
// t+768); warp 0 merges eight each (l, l+32, ..., l+224), then by butterfly, and stores the
// CTA total into slot `me` of every CTA (DSMEM); after the cluster barrier warp 0 merges
// the cs <= 16 slots in rank order.  One cluster barrier and two __syncthreads; slots
// [2][NV][16] are double-buffered by `parity`.
template <int NV>
__device__ __forceinline__ void cluster_reduce_tree(const ff (&acc)[NV], ff (&out)[NV], ff* sbuf, ff* slots,
                                                    unsigned parity, unsigned me, unsigned cs) {
    static_assert(CBS == 1024, "the tree assumes 1024 threads");
    const int t = threadIdx.x;
#pragma unroll
    for (int i = 0; i < NV; ++i) sbuf[i * CBS + t] = acc[i];
    __syncthreads();
    if (t < 256) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            ff x = sbuf[i * CBS + t];
            ff_merge(x, sbuf[i * CBS + t + 256]);
            ff_merge(x, sbuf[i * CBS + t + 512]);
            ff_merge(x, sbuf[i * CBS + t + 768]);
            sbuf[i * CBS + t] = x;  // only thread t reads or writes position t in this stage
        }
    }
    __syncthreads();
    if (t < 32) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            ff x = sbuf[i * CBS + t];
#pragma unroll
            for (int k = 1; k < 8; ++k) ff_merge(x, sbuf[i * CBS + t + 32 * k]);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) ff_shfl_merge(x, o);
            if ((unsigned)t < cs) st_cluster_v2f32(map_rank(slots + (parity * NV + i) * 16 + me, t), x.hi, x.lo);
        }
    }
    cluster_sync_all();
    if (t < 32) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            ff y = (unsigned)t < cs ? slots[(parity * NV + i) * 16 + t] : ff_zero();
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) ff_shfl_merge(y, o);
            if (t == 0) out[i] = y;
        }
    }
}

}  // namespace wcfd
