// Cluster-resident CG: one thread-block cluster (up to 16 CTAs) holds the whole scalar
// system in shared memory for the length of the solve.
//
//  * CTA q of the cluster owns rows [q R, (q+1) R); its slice of the matrix (off-diagonals,
//    packed (rank, local) columns, diagonal) and of every vector lives in its shared memory.
//  * A neighbour value owned by another CTA is read through distributed shared memory
//    (mapa + ld.shared::cluster); nothing touches global memory between the set-up and
//    the final write of x.
//  * Grid-wide synchronisation is the hardware cluster barrier
//    (barrier.cluster.arrive.release / wait.acquire).  A dot product is an all-reduce: each
//    CTA sums its rows (exact products in float-float, common.cuh), stores its fp64 total
//    into a slot of every CTA's shared memory, and after the barrier one warp per CTA adds
//    the CS slots in a fixed order, so all CTAs (and all runs) agree bit for bit.  All CTAs take the same branch at every test, so no CTA can
//    leave while another still waits or reads its memory.
//  * The direction update p = z + beta p is evaluated inside the SpMV for the row and its
//    neighbours (double-buffered p), so an iteration needs two barriers.
// The arithmetic is that of cg_kernel (krylov.cu): the same Jacobi-preconditioned CG with
// fp64 dot products and the same stop test.
#include "common.cuh"
#include "kernels.cuh"

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

// dynamic shared memory per CTA for R rows and width W:
// off + packed columns (8 W) and diag, invd, x, r, p (two buffers), q (28)
size_t cluster_cg_smem_bytes(int R, int W) { return (size_t)R * (8 * (size_t)W + 28); }

template <int W>
__global__ void __launch_bounds__(CBS) cg_cluster_kernel(KrylovArgs a, int R) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ ff slots[2 * 2 * 16];
    struct Scal {
        double rr, rz;
        float af, bf;
        int go, status, k;
    };
    __shared__ Scal sc;
    const int C = a.m.n_cells;
    const unsigned me = cluster_rank();
    const unsigned cs = cluster_nranks();
    const int row0 = (int)me * R;
    const int nloc = max(0, min(R, C - row0));
    float* off = reinterpret_cast<float*>(smem);                 // [W][R]
    uint32_t* colp = reinterpret_cast<uint32_t*>(off + (size_t)W * R);  // [W][R] (rank << 24) | local
    float* diag = reinterpret_cast<float*>(colp + (size_t)W * R);
    float* invd = diag + R;
    float* x = invd + R;
    float* r = x + R;
    float* pbuf0 = r + R;
    float* pbuf1 = pbuf0 + R;
    float* q = pbuf1 + R;

    // load this CTA's slice
    for (int l = threadIdx.x; l < nloc; l += CBS) {
        const int g = row0 + l;
        diag[l] = a.A.diag[g];
        invd[l] = diag[l] != 0.0f ? 1.0f / diag[l] : 1.0f;
        x[l] = a.x[g];
#pragma unroll
        for (int j = 0; j < W; ++j) {
            off[(size_t)j * R + l] = a.A.off[(size_t)j * C + g];
            const int c = a.m.ell_col[(size_t)j * C + g];
            const int rk = c / R;
            colp[(size_t)j * R + l] = ((uint32_t)rk << 24) | (uint32_t)(c - rk * R);
        }
    }
    cluster_sync_all();
    // r = b - A x ; p = z = M r ; rr ; rz
    ff acc[2] = {ff_zero(), ff_zero()};
    for (int l = threadIdx.x; l < nloc; l += CBS) {
        float ax = diag[l] * x[l];
#pragma unroll
        for (int j = 0; j < W; ++j) ax += off[(size_t)j * R + l] * ld_col(x, colp[(size_t)j * R + l], me);
        const float ri = a.A.rhs[row0 + l] - ax;
        const float zi = ri * invd[l];
        r[l] = ri;
        pbuf0[l] = zi;
        ff_fma(acc[0], ri, ri);
        ff_fma(acc[1], ri, zi);
    }
    unsigned parity = 0;
    double red[2];
    cluster_allreduce<2>(acc, red, slots, parity, me, cs);
    parity ^= 1u;
    // fp64 scalar work by thread 0 only (fp64 runs at ~1/64 of the fp32 rate on GB300)
    if (threadIdx.x == 0) {
        sc.rr = red[0];
        sc.rz = red[1];
        sc.bf = 0.0f;
        sc.k = 0;
        sc.status = WCFD_OK;
        sc.go = (0 < a.maxiter && red[0] > a.atol2);
    }
    __syncthreads();
    int cur = 0;
    while (sc.go) {
        const float bf = sc.bf;
        float* po = cur ? pbuf1 : pbuf0;
        float* pn = cur ? pbuf0 : pbuf1;
        ff accq[1] = {ff_zero()};
        for (int l = threadIdx.x; l < nloc; l += CBS) {
            const float pi = r[l] * invd[l] + bf * po[l];
            float qi = diag[l] * pi;
#pragma unroll
            for (int j = 0; j < W; ++j) {
                const uint32_t cp = colp[(size_t)j * R + l];
                const float rc = ld_col(r, cp, me);
                const float dc = ld_col(invd, cp, me);
                const float pc = ld_col(po, cp, me);
                qi += off[(size_t)j * R + l] * (rc * dc + bf * pc);
            }
            pn[l] = pi;
            q[l] = qi;
            ff_fma(accq[0], pi, qi);
        }
        double pq[1];
        cluster_allreduce<1>(accq, pq, slots, parity, me, cs);
        parity ^= 1u;
        if (threadIdx.x == 0) {
            if (pq[0] == 0.0) {
                sc.status = WCFD_KRYLOV_BREAKDOWN;
                sc.go = 0;
            } else {
                sc.af = (float)(sc.rz / pq[0]);
            }
        }
        __syncthreads();
        if (!sc.go) break;
        const float af = sc.af;
        ff acc2[2] = {ff_zero(), ff_zero()};
        for (int l = threadIdx.x; l < nloc; l += CBS) {
            x[l] += af * pn[l];
            const float ri = r[l] - af * q[l];
            r[l] = ri;
            const float zi = ri * invd[l];
            ff_fma(acc2[0], ri, ri);
            ff_fma(acc2[1], ri, zi);
        }
        double red2[2];
        cluster_allreduce<2>(acc2, red2, slots, parity, me, cs);
        parity ^= 1u;
        if (threadIdx.x == 0) {
            sc.rr = red2[0];
            sc.bf = (float)(sc.rz != 0.0 ? red2[1] / sc.rz : 0.0);
            sc.rz = red2[1];
            sc.k += 1;
            sc.go = (sc.k < a.maxiter && sc.rr > a.atol2);
        }
        __syncthreads();
        cur ^= 1;
    }
    for (int l = threadIdx.x; l < nloc; l += CBS) a.x[row0 + l] = x[l];
    if (me == 0 && threadIdx.x == 0) {
        int st = sc.status;
        if (st == WCFD_OK && !(sc.rr <= a.atol2)) st = WCFD_NOT_CONVERGED;
        a.stats->iterations = sc.k;
        a.stats->status = st;
        a.stats->residual = sqrt(sc.rr);
    }
}

const void* cg_cluster_kernel_for(int W) {
    switch (W) {
        case 0: return (const void*)cg_cluster_kernel<0>;
        case 1: return (const void*)cg_cluster_kernel<1>;
        case 2: return (const void*)cg_cluster_kernel<2>;
        case 3: return (const void*)cg_cluster_kernel<3>;
        case 4: return (const void*)cg_cluster_kernel<4>;
        case 5: return (const void*)cg_cluster_kernel<5>;
        case 6: return (const void*)cg_cluster_kernel<6>;
        default: return nullptr;
    }
}

}  // namespace wcfd
