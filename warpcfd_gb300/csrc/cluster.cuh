// Thread-block-cluster primitives shared by the cluster-resident solvers: rank queries,
// the hardware cluster barrier, distributed-shared-memory loads and stores, and a
// deterministic float-float reduction over the CTAs of a cluster.
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
// The cluster barrier of a reduction: warp 0 (which made the remote slot stores) arrives
// with release semantics, the other warps arrive relaxed, every thread waits with acquire.
// Everything the other warps wrote before the CTA's last __syncthreads happens before
// warp 0's release (the CTA barrier orders it, and the release is cumulative), so the
// other CTAs see it after their wait; a release by 32 instead of 1,024 threads.
__device__ __forceinline__ void cluster_sync_warp0_release() {
    if (threadIdx.x < 32)
        asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
    else
        asm volatile("barrier.cluster.arrive.relaxed.aligned;" ::: "memory");
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
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
__device__ __forceinline__ float4 ld_cluster_f32x4(uint32_t addr) {
    float4 v;
    asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(addr));
    return v;
}
__device__ __forceinline__ void st_cluster_v2f32(uint32_t addr, float a, float b) {
    asm volatile("st.shared::cluster.v2.f32 [%0], {%1, %2};" :: "r"(addr), "f"(a), "f"(b) : "memory");
}

// Sum NV float-float values over the CTAs of the cluster, result (float-float, the same bits
// in every CTA) in thread 0 only.  The block stage is a shared-memory tree instead of a
// butterfly in every warp, so that most warps issue one store and wait: every thread
// stores its values into sbuf [NV][CBS]; threads 0..255 merge four each ((t + t+256) +
// (t+512 + t+768), a pairwise tree so the merges overlap); warp 0 merges eight each
// (l, l+32, ..., l+224, again pairwise), then by butterfly, and stores the CTA total into
// slot `me` of every CTA (DSMEM); after the cluster barrier (release by warp 0 only)
// warp 0 merges the cs <= 16 slots in rank order (four butterfly levels).  One cluster
// barrier and two __syncthreads; slots [2][NV][16] are double-buffered by `parity`.
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
            const ff* b = sbuf + i * CBS + t;
            ff x0 = b[0], x1 = b[256], x2 = b[512], x3 = b[768];
            ff_merge(x0, x1);
            ff_merge(x2, x3);
            ff_merge(x0, x2);
            sbuf[i * CBS + t] = x0;  // only thread t reads or writes position t in this stage
        }
    }
    __syncthreads();
    if (t < 32) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            const ff* b = sbuf + i * CBS + t;
            ff y[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) y[k] = b[32 * k];
#pragma unroll
            for (int k = 0; k < 8; k += 2) ff_merge(y[k], y[k + 1]);
            ff_merge(y[0], y[2]);
            ff_merge(y[4], y[6]);
            ff_merge(y[0], y[4]);
            ff x = y[0];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) ff_shfl_merge(x, o);
            if ((unsigned)t < cs) st_cluster_v2f32(map_rank(slots + (parity * NV + i) * 16 + me, t), x.hi, x.lo);
        }
    }
    cluster_sync_warp0_release();
    if (t < 32) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            ff y = (unsigned)t < cs ? slots[(parity * NV + i) * 16 + t] : ff_zero();
#pragma unroll
            for (int o = 8; o > 0; o >>= 1) ff_shfl_merge(y, o);  // lanes 0..15 hold the cs <= 16 slots
            if (t == 0) out[i] = y;
        }
    }
}

}  // namespace wcfd
