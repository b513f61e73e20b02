// Cluster-resident CG: one thread-block cluster (up to 16 CTAs) holds the whole scalar
// system in shared memory for the length of the solve.
//
//  * CTA q of the cluster owns rows [q R, (q+1) R); its slice of the matrix (off-diagonals,
//    packed (rank, local) columns, diagonal) and the gathered vectors (z and p, stored as
//    (z, p) pairs so one 8-byte load fetches both) live in its shared memory; x, r and q of
//    a thread's own rows stay in registers.
//  * A neighbour value owned by another CTA is read through distributed shared memory
//    (mapa + ld.shared::cluster); nothing touches global memory between the set-up and
//    the final write of x.
//  * Grid-wide synchronisation is the hardware cluster barrier
//    (barrier.cluster.arrive.release / wait.acquire).  A dot product is reduced by a
//    shared-memory tree in each CTA (exact products in float-float, common.cuh); warp 0
//    stores the CTA total into a slot of every CTA's shared memory and after the barrier
//    merges the cs slots in a fixed order, so all CTAs (and all runs) agree bit for bit.
//    Thread 0 forms alpha and beta from the float-float sums and broadcasts them.  All
//    CTAs take the same branch at every test, so no CTA can leave while another still
//    waits or reads its memory.
//  * The direction update p = z + beta p is evaluated inside the SpMV for the row and its
//    neighbours (double-buffered p), so an iteration needs two barriers.
// The arithmetic is that of cg_kernel (krylov.cu): the same Jacobi-preconditioned CG with
// fp64-accurate dot products and the same stop test.
#include "cluster.cuh"
#include "common.cuh"
#include "kernels.cuh"

namespace wcfd {

// Dynamic shared memory per CTA for R rows and width W: the reduction tree (3 x 1024
// float-float values), then per row the pairs (z, p) of two iteration buffers (16), the
// off-diagonals (4 W), diag and 1/diag (8) and 16-bit packed columns (2 W).  x, r and q
// live in registers (each thread owns the same rows for the whole solve).  16 CTAs of
// R <= 4096 rows hold 65536 rows of width 4.
size_t cluster_cg_smem_bytes(int R, int W) {
    return 3 * (size_t)CBS * sizeof(ff) + (size_t)R * (6 * (size_t)W + 24);
}

// largest R whose shared memory fits `optin` bytes per CTA (capped by the 12-bit local
// index of the packed columns)
int cluster_cg_max_rows(int W, int optin) {
    const long long fixed = 3LL * CBS * (long long)sizeof(ff) + 2048;  // tree + static shared memory
    long long r = ((long long)optin - fixed) / (6LL * W + 24);
    if (r > 4096) r = 4096;
    return r > 0 ? (int)r : 0;
}

// rows per thread for R rows per CTA
int cluster_cg_rpt(int R) { return R <= CBS ? 1 : (R <= 2 * CBS ? 2 : 4); }

__device__ __forceinline__ float2 ld_cluster_f32x2(uint32_t addr) {
    float2 v;
    asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr));
    return v;
}

template <int W, int RPT>
__device__ __forceinline__ void cg_cluster_body(const KrylovArgs& a, int R) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ ff slots[2 * 3 * 16];
    __shared__ unsigned char chunk_local[4096 / 32];  // 32-row chunk with no off-CTA neighbour
    struct Scal {
        ff rr, rz, pq, thr2;
        float af, bf;
        int go, status, k;
    };
    __shared__ Scal sc;
    const int C = a.m.n_cells;
    const unsigned me = cluster_rank();
    const unsigned cs = cluster_nranks();
    const int row0 = (int)me * R;
    const int nloc = max(0, min(R, C - row0));
    ff* sbuf = reinterpret_cast<ff*>(smem);                               // [3][CBS]
    float2* zp0 = reinterpret_cast<float2*>(sbuf + 3 * CBS);              // [R] (z, p) of buffer 0
    float2* zp1 = zp0 + R;                                                // [R] buffer 1
    float* off = reinterpret_cast<float*>(zp1 + R);                       // [W][R]
    float* diag = off + W * R;
    float* invd = diag + R;
    uint16_t* colp = reinterpret_cast<uint16_t*>(invd + R);              // [W][R] (rank << 12) | local
    const int t0 = threadIdx.x;

    // this CTA's slice of the matrix
    for (int l = t0; l < nloc; l += CBS) {
        const int g = row0 + l;
        const float d = a.A.diag[g];
        diag[l] = d;
        invd[l] = d != 0.0f ? 1.0f / d : 1.0f;
        bool local = true;
#pragma unroll
        for (int j = 0; j < W; ++j) {
            off[j * R + l] = a.A.off[(size_t)j * C + g];
            const int c = a.m.ell_col[(size_t)j * C + g];
            const int rk = c / R;
            colp[j * R + l] = (uint16_t)((rk << 12) | (c - rk * R));
            local = local && rk == (int)me;
        }
        // a warp's lanes hold the 32 consecutive rows of one chunk, here and in the passes
        local = __all_sync(__activemask(), local);
        if ((t0 & 31) == 0) chunk_local[l >> 5] = local ? 1 : 0;
    }
    // own rows l = t0 + u CBS, u < RPT: x, r, q, p in registers
    float xr[RPT], rr_[RPT], qr[RPT], pr[RPT];
    // r = b - A x (x read from global) ; z = M r ; first direction p = z (the p half of
    // buffer 0 is zero and beta 0) ; rr ; rz ; bb
    ff acc[3] = {ff_zero(), ff_zero(), ff_zero()};
#pragma unroll
    for (int u = 0; u < RPT; ++u) {
        const int l = t0 + u * CBS;
        xr[u] = 0.0f;
        rr_[u] = 0.0f;
        qr[u] = 0.0f;
        pr[u] = 0.0f;
        if (l < nloc) {
            const int g = row0 + l;
            xr[u] = a.x[g];
            float ax = diag[l] * xr[u];
#pragma unroll
            for (int j = 0; j < W; ++j) ax += off[j * R + l] * a.x[a.m.ell_col[(size_t)j * C + g]];
            const float bi = a.A.rhs[g];
            const float ri = bi - ax;
            const float zi = ri * invd[l];
            rr_[u] = ri;
            zp0[l] = make_float2(zi, 0.0f);
            ff_fma(acc[0], ri, ri);
            ff_fma(acc[1], ri, zi);
            ff_fma(acc[2], bi, bi);
        }
    }
    unsigned parity = 0;
    ff red[3];
    cluster_reduce_tree<3>(acc, red, sbuf, slots, parity, me, cs);
    parity ^= 1u;
    if (t0 == 0) {
        const double rr0 = ff_to_double(red[0]);
        sc.rr = ff_norm(red[0]);
        sc.rz = ff_norm(red[1]);
        sc.thr2 = ff_norm(ff_from_double(fmax(a.atol2, a.rtol2 * rr0)));
        sc.bf = 0.0f;
        sc.k = 0;
        sc.status = WCFD_OK;
        sc.go = (0 < a.maxiter && ff_gt(sc.rr, sc.thr2));
        if (me == 0) {
            a.stats->initial_residual = sqrt(rr0);
            a.stats->rhs_norm = sqrt(ff_to_double(red[2]));
        }
    }
    __syncthreads();
    int cur = 0;
    while (sc.go) {
        const float bf = sc.bf;
        // buffer cur holds (z_k, p_{k-1}); p_k and then z_{k+1} go to the other buffer
        const float2* zpo = cur ? zp1 : zp0;
        float2* zpn = cur ? zp0 : zp1;
        // p = z + beta p_old (own row and each neighbour) ; q = A p ; p.q
        ff accq[1] = {ff_zero()};
#pragma unroll
        for (int u = 0; u < RPT; ++u) {
            const int l = t0 + u * CBS;
            if (l < nloc) {
                const float2 own = zpo[l];
                const float pi = own.x + bf * own.y;
                float qi = diag[l] * pi;
                if (chunk_local[l >> 5]) {  // warp-uniform: every neighbour in this CTA
#pragma unroll
                    for (int j = 0; j < W; ++j) {
                        const float2 v = zpo[colp[j * R + l] & 0xFFFu];
                        qi += off[j * R + l] * (v.x + bf * v.y);
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < W; ++j) {
                        const unsigned cp = colp[j * R + l];
                        const unsigned rk = cp >> 12;
                        const unsigned lo = cp & 0xFFFu;
                        const float2 v = rk == me ? zpo[lo] : ld_cluster_f32x2(map_rank(zpo + lo, rk));
                        qi += off[j * R + l] * (v.x + bf * v.y);
                    }
                }
                zpn[l].y = pi;
                pr[u] = pi;
                qr[u] = qi;
                ff_fma(accq[0], pi, qi);
            }
        }
        ff pq[1];
        cluster_reduce_tree<1>(accq, pq, sbuf, slots, parity, me, cs);
        parity ^= 1u;
        if (t0 == 0) {
            const ff pqn = ff_norm(pq[0]);
            if (pqn.hi == 0.0f) {
                sc.status = WCFD_KRYLOV_BREAKDOWN;
                sc.go = 0;
            } else {
                sc.af = ff_div_to_float(sc.rz, pqn);
            }
        }
        __syncthreads();
        if (!sc.go) break;
        const float af = sc.af;
        // x += alpha p ; r -= alpha q ; z = M r ; rr ; rz
        ff acc2[2] = {ff_zero(), ff_zero()};
#pragma unroll
        for (int u = 0; u < RPT; ++u) {
            const int l = t0 + u * CBS;
            if (l < nloc) {
                xr[u] += af * pr[u];
                const float ri = rr_[u] - af * qr[u];
                const float zi = ri * invd[l];
                rr_[u] = ri;
                zpn[l].x = zi;
                ff_fma(acc2[0], ri, ri);
                ff_fma(acc2[1], ri, zi);
            }
        }
        ff red2[2];
        cluster_reduce_tree<2>(acc2, red2, sbuf, slots, parity, me, cs);
        parity ^= 1u;
        if (t0 == 0) {
            const ff rzn = ff_norm(red2[1]);
            sc.rr = ff_norm(red2[0]);
            sc.bf = sc.rz.hi != 0.0f ? ff_div_to_float(rzn, sc.rz) : 0.0f;
            sc.rz = rzn;
            sc.k += 1;
            sc.go = (sc.k < a.maxiter && ff_gt(sc.rr, sc.thr2));
        }
        __syncthreads();
        cur ^= 1;
    }
#pragma unroll
    for (int u = 0; u < RPT; ++u) {
        const int l = t0 + u * CBS;
        if (l < nloc) a.x[row0 + l] = xr[u];
    }
    if (me == 0 && t0 == 0) {
        int st = sc.status;
        if (st == WCFD_OK && !ff_le(sc.rr, sc.thr2)) st = WCFD_NOT_CONVERGED;
        a.stats->iterations = sc.k;
        a.stats->status = st;
        a.stats->residual = sqrt(ff_to_double(sc.rr));
    }
}

template <int W, int RPT>
__global__ void __launch_bounds__(CBS) cg_cluster_kernel(KrylovArgs a, int R) {
    cg_cluster_body<W, RPT>(a, R);
}

// One cluster per case of a device case table: the pressure CG of every case
// (pres system, p_x warm start, stats[1]), cs CTAs per cluster.  refine = 1 solves a
// refinement sweep's correction instead: right-hand side p_work[0, C) (the fp64 residual
// rounded once), solution p_work[C, 2C) from zero, relative stop p_refine_rtol.
template <int W, int RPT>
__global__ void __launch_bounds__(CBS) cg_cluster_batched(const wcfd_case* __restrict__ cases, int cs, int refine) {
    const wcfd_case& c = cases[blockIdx.x / cs];
    KrylovArgs a = {};
    a.m = c.mesh;
    a.A = c.pres;
    a.x = c.p_x;
    a.atol2 = c.prm.atol_p * c.prm.atol_p;
    a.rtol2 = c.prm.rtol_p * c.prm.rtol_p;
    if (refine) {
        a.A.rhs = c.p_work;
        a.x = c.p_work + c.mesh.n_cells;
        a.atol2 = 0.0;
        a.rtol2 = c.prm.p_refine_rtol * c.prm.p_refine_rtol;
    }
    a.maxiter = c.prm.maxiter;
    a.stats = c.stats + 1;
    cg_cluster_body<W, RPT>(a, (c.mesh.n_cells + cs - 1) / cs);
}

// BiCGSTAB on one case per cluster, for the batched form: the momentum system of the
// case (interleaved 3C rows, shared off-diagonals) with its vectors in global memory
// (the case's workspace: r, r0, pA, pB, vA, vB, t, s, invd), rows spread over the cluster's
// CTAs, hardware cluster barriers and the DSMEM all-reduce.  Values written by another CTA
// during the solve are read through L2 (ld.cg).  Same algorithm and arithmetic as
// bicgstab_kernel (krylov.cu).
template <int W>
__device__ __forceinline__ void bicgstab_cluster_body(const wcfd_case& cse) {
    __shared__ ff slots[2 * 3 * 16];
    __shared__ ff sbuf[2 * CBS];
    struct Scal {
        ff rr, rho, alpha, omega, thr2;
        float af, bf, of;
        int go, status, k;
    };
    __shared__ Scal sc;
    const unsigned me = cluster_rank();
    const unsigned cs = cluster_nranks();
    const int C = cse.mesh.n_cells;
    const size_t n3 = 3 * (size_t)C;
    float* ws = cse.ws_u.vec;
    float* r = ws;
    float* r0 = ws + n3;
    float* pbuf[2] = {ws + 2 * n3, ws + 3 * n3};
    float* vbuf[2] = {ws + 4 * n3, ws + 5 * n3};
    float* t = ws + 6 * n3;
    float* s = ws + 7 * n3;
    float* invd = ws + 8 * n3;
    const float* __restrict__ b = cse.mom.rhs;
    const float* __restrict__ diag = cse.mom.diag;
    const float* __restrict__ off = cse.mom.off;
    const int* __restrict__ col = cse.mesh.ell_col;
    float* x = cse.hbya;
    const double atol2 = cse.prm.atol_u * cse.prm.atol_u;
    const double rtol2 = cse.prm.rtol_u * cse.prm.rtol_u;
    const int maxiter = cse.prm.maxiter;
    const int stride = (int)cs * CBS;
    const int i0 = (int)me * CBS + threadIdx.x;
    unsigned parity = 0;

    ff acc[2] = {ff_zero(), ff_zero()};
    for (int i = i0; i < C; i += stride) {
        float ax[3];
#pragma unroll
        for (int o = 0; o < 3; ++o) ax[o] = diag[3 * (size_t)i + o] * x[3 * (size_t)i + o];
#pragma unroll
        for (int j = 0; j < W; ++j) {
            const float v = off[(size_t)j * C + i];
            const int c = col[(size_t)j * C + i];
#pragma unroll
            for (int o = 0; o < 3; ++o) ax[o] += v * x[3 * (size_t)c + o];
        }
#pragma unroll
        for (int o = 0; o < 3; ++o) {
            const size_t q = 3 * (size_t)i + o;
            const float ri = b[q] - ax[o];
            r[q] = ri;
            r0[q] = ri;
            pbuf[0][q] = ri;
            vbuf[0][q] = 0.0f;
            invd[q] = diag[q] != 0.0f ? 1.0f / diag[q] : 1.0f;
            ff_fma(acc[0], ri, ri);
            ff_fma(acc[1], b[q], b[q]);
        }
    }
    ff red[2];
    cluster_reduce_tree<2>(acc, red, sbuf, slots, parity, me, cs);
    parity ^= 1u;
    if (threadIdx.x == 0) {
        const double rr0 = ff_to_double(red[0]);
        sc.rr = ff_norm(red[0]);
        sc.rho = sc.rr;
        sc.thr2 = ff_norm(ff_from_double(fmax(atol2, rtol2 * rr0)));
        sc.bf = 0.0f;
        sc.of = 0.0f;
        sc.k = 0;
        sc.status = WCFD_OK;
        sc.go = (0 < maxiter && ff_gt(sc.rr, sc.thr2));
        if (me == 0) {
            cse.stats[0].initial_residual = sqrt(rr0);
            cse.stats[0].rhs_norm = sqrt(ff_to_double(red[1]));
        }
    }
    __syncthreads();
    int cur = 0;
    while (sc.go) {
        const float bf = sc.bf, of0 = sc.of;
        const float* po = pbuf[cur];
        const float* vo = vbuf[cur];
        float* pn = pbuf[cur ^ 1];
        float* vn = vbuf[cur ^ 1];
        ff accv[1] = {ff_zero()};
        for (int i = i0; i < C; i += stride) {
            float pi[3], vi[3];
#pragma unroll
            for (int o = 0; o < 3; ++o) {
                const size_t q = 3 * (size_t)i + o;
                pi[o] = __ldcg(r + q) + bf * (__ldcg(po + q) - of0 * __ldcg(vo + q));
                vi[o] = diag[q] * (pi[o] * __ldcg(invd + q));
            }
#pragma unroll
            for (int j = 0; j < W; ++j) {
                const float v = off[(size_t)j * C + i];
                const int c = col[(size_t)j * C + i];
#pragma unroll
                for (int o = 0; o < 3; ++o) {
                    const size_t q = 3 * (size_t)c + o;
                    const float pc = __ldcg(r + q) + bf * (__ldcg(po + q) - of0 * __ldcg(vo + q));
                    vi[o] += v * (pc * __ldcg(invd + q));
                }
            }
#pragma unroll
            for (int o = 0; o < 3; ++o) {
                const size_t q = 3 * (size_t)i + o;
                pn[q] = pi[o];
                vn[q] = vi[o];
                ff_fma(accv[0], r0[q], vi[o]);
            }
        }
        ff r0v[1];
        cluster_reduce_tree<1>(accv, r0v, sbuf, slots, parity, me, cs);
        parity ^= 1u;
        if (threadIdx.x == 0) {
            const ff d = ff_norm(r0v[0]);
            if (d.hi == 0.0f) {
                sc.status = WCFD_KRYLOV_BREAKDOWN;
                sc.go = 0;
            } else {
                sc.alpha = ff_div(sc.rho, d);
                sc.af = ff_to_float(sc.alpha);
            }
        }
        __syncthreads();
        if (!sc.go) break;
        const float af = sc.af;
        ff acct[2] = {ff_zero(), ff_zero()};
        for (int i = i0; i < C; i += stride) {
            float si[3], ti[3];
#pragma unroll
            for (int o = 0; o < 3; ++o) {
                const size_t q = 3 * (size_t)i + o;
                si[o] = __ldcg(r + q) - af * __ldcg(vn + q);
                x[q] += af * (pn[q] * invd[q]);
                ti[o] = diag[q] * (si[o] * invd[q]);
            }
#pragma unroll
            for (int j = 0; j < W; ++j) {
                const float v = off[(size_t)j * C + i];
                const int c = col[(size_t)j * C + i];
#pragma unroll
                for (int o = 0; o < 3; ++o) {
                    const size_t q = 3 * (size_t)c + o;
                    const float scv = __ldcg(r + q) - af * __ldcg(vn + q);
                    ti[o] += v * (scv * __ldcg(invd + q));
                }
            }
#pragma unroll
            for (int o = 0; o < 3; ++o) {
                const size_t q = 3 * (size_t)i + o;
                s[q] = si[o];
                t[q] = ti[o];
                ff_fma(acct[0], ti[o], ti[o]);
                ff_fma(acct[1], ti[o], si[o]);
            }
        }
        ff ts[2];
        cluster_reduce_tree<2>(acct, ts, sbuf, slots, parity, me, cs);
        parity ^= 1u;
        if (threadIdx.x == 0) {
            const ff tt = ff_norm(ts[0]);
            sc.omega = tt.hi != 0.0f ? ff_div(ts[1], tt) : ff_zero();
            sc.of = ff_to_float(sc.omega);
        }
        __syncthreads();
        const float of = sc.of;
        ff accr[2] = {ff_zero(), ff_zero()};
        for (int i = i0; i < C; i += stride) {
#pragma unroll
            for (int o = 0; o < 3; ++o) {
                const size_t q = 3 * (size_t)i + o;
                const float si = s[q];
                x[q] += of * (si * invd[q]);
                const float ri = si - of * t[q];
                r[q] = ri;
                ff_fma(accr[0], ri, ri);
                ff_fma(accr[1], r0[q], ri);
            }
        }
        ff rr2[2];
        cluster_reduce_tree<2>(accr, rr2, sbuf, slots, parity, me, cs);
        parity ^= 1u;
        if (threadIdx.x == 0) {
            sc.rr = ff_norm(rr2[0]);
            sc.k += 1;
            if (sc.omega.hi == 0.0f || sc.rho.hi == 0.0f) {
                sc.status = WCFD_KRYLOV_BREAKDOWN;
                sc.go = 0;
            } else {
                const ff rho_n = ff_norm(rr2[1]);
                sc.bf = ff_to_float(ff_mul(ff_div(rho_n, sc.rho), ff_div(sc.alpha, sc.omega)));
                sc.rho = rho_n;
                sc.go = (sc.k < maxiter && ff_gt(sc.rr, sc.thr2));
            }
        }
        __syncthreads();
        cur ^= 1;
    }
    if (me == 0 && threadIdx.x == 0) {
        int st = sc.status;
        if (st == WCFD_OK && !ff_le(sc.rr, sc.thr2)) st = WCFD_NOT_CONVERGED;
        cse.stats[0].iterations = sc.k;
        cse.stats[0].status = st;
        cse.stats[0].residual = sqrt(ff_to_double(sc.rr));
    }
}

template <int W>
__global__ void __launch_bounds__(CBS) bicgstab_cluster_batched(const wcfd_case* __restrict__ cases, int cs_req) {
    bicgstab_cluster_body<W>(cases[blockIdx.x / cs_req]);
}

#define WCFD_W_SWITCH(NAME)                      \
    switch (W) {                                 \
        case 0: return (const void*)NAME<0>;     \
        case 1: return (const void*)NAME<1>;     \
        case 2: return (const void*)NAME<2>;     \
        case 3: return (const void*)NAME<3>;     \
        case 4: return (const void*)NAME<4>;     \
        case 5: return (const void*)NAME<5>;     \
        case 6: return (const void*)NAME<6>;     \
        default: return nullptr;                 \
    }

#define WCFD_WR_SWITCH(NAME)                                   \
    switch (W * 8 + cluster_cg_rpt(R)) {                       \
        case 0 * 8 + 1: return (const void*)NAME<0, 1>;        \
        case 0 * 8 + 2: return (const void*)NAME<0, 2>;        \
        case 0 * 8 + 4: return (const void*)NAME<0, 4>;        \
        case 1 * 8 + 1: return (const void*)NAME<1, 1>;        \
        case 1 * 8 + 2: return (const void*)NAME<1, 2>;        \
        case 1 * 8 + 4: return (const void*)NAME<1, 4>;        \
        case 2 * 8 + 1: return (const void*)NAME<2, 1>;        \
        case 2 * 8 + 2: return (const void*)NAME<2, 2>;        \
        case 2 * 8 + 4: return (const void*)NAME<2, 4>;        \
        case 3 * 8 + 1: return (const void*)NAME<3, 1>;        \
        case 3 * 8 + 2: return (const void*)NAME<3, 2>;        \
        case 3 * 8 + 4: return (const void*)NAME<3, 4>;        \
        case 4 * 8 + 1: return (const void*)NAME<4, 1>;        \
        case 4 * 8 + 2: return (const void*)NAME<4, 2>;        \
        case 4 * 8 + 4: return (const void*)NAME<4, 4>;        \
        case 5 * 8 + 1: return (const void*)NAME<5, 1>;        \
        case 5 * 8 + 2: return (const void*)NAME<5, 2>;        \
        case 5 * 8 + 4: return (const void*)NAME<5, 4>;        \
        case 6 * 8 + 1: return (const void*)NAME<6, 1>;        \
        case 6 * 8 + 2: return (const void*)NAME<6, 2>;        \
        case 6 * 8 + 4: return (const void*)NAME<6, 4>;        \
        default: return nullptr;                               \
    }

const void* cg_cluster_batched_for(int W, int R) { WCFD_WR_SWITCH(cg_cluster_batched) }
const void* bicgstab_cluster_batched_for(int W) { WCFD_W_SWITCH(bicgstab_cluster_batched) }
const void* cg_cluster_kernel_for(int W, int R) { WCFD_WR_SWITCH(cg_cluster_kernel) }

}  // namespace wcfd
