// Single-reduction cluster-resident CG (Chronopoulos and Gear, "s-step iterative methods
// for symmetric linear systems", J. Comput. Appl. Math. 25 (1989), the one-reduction
// rearrangement of Jacobi-preconditioned CG), one thread-block cluster per system.
//
// Textbook CG needs two all-reduces per iteration (p.q for alpha, then r.z for beta); on a
// cluster each costs a shared-memory tree, a release/acquire cluster barrier and a
// broadcast, about 2,000 cycles, which is most of an iteration of a system that lives in
// shared memory.  This form carries w = A u (u = M r) and s = A p by recurrence and takes
// gamma = r.u, delta = w.u and r.r from ONE all-reduce:
//
//     beta_i  = gamma_i / gamma_{i-1}
//     alpha_i = gamma_i / (delta_i - beta_i gamma_i / alpha_{i-1})      (= gamma_i / p_i.A p_i)
//     p = u + beta p ;  s = w + beta s ;  x += alpha p ;  r -= alpha s ;  u = M r ;  w = A u
//
// All of an iteration runs in one pass over the rows between two all-reduces: the SpMV
// w = A u needs the new u of every neighbour, which is formed on the fly from the
// neighbour's previous r, w, s (u_c = (r_c - alpha (w_c + beta s_c)) / d_c), read as one
// 16-byte record (r, w, s, 1/d) from a double buffer in shared memory (DSMEM for another
// CTA's rows).  The iterates are those of textbook CG in exact arithmetic; in floating
// point they differ at rounding level.  Same stop test as cg_kernel: ||r_i|| <= atol (or
// rtol ||r_0||) before iteration i, at most maxiter updates of x.
//
// Registers hold x, p, s, r, u, w of a thread's own rows (RPT <= 2 rows per thread).
#include "cluster.cuh"
#include "common.cuh"
#include "kernels.cuh"

namespace wcfd {

// dynamic shared memory: the reduction tree (3 x 1024 float-float), two (r, w, s, 1/d)
// buffers (32), off-diagonals (4 W), diag (4) and 16-bit packed columns (2 W) per row
size_t cluster_cg1_smem_bytes(int R, int W) {
    return 3 * (size_t)CBS * sizeof(ff) + (size_t)R * (6 * (size_t)W + 36);
}

template <int W, int RPT>
__device__ __forceinline__ void cg1_cluster_body(const KrylovArgs& a, int R) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ ff slots[2 * 3 * 16];
    __shared__ unsigned char chunk_local[4096 / 32];  // 32-row chunk with no off-CTA neighbour
    struct Scal {
        ff rr, gamma, thr2;
        float af, bf, alpha_prev;
        int go, status, k;
    };
    __shared__ Scal sc;
    const int C = a.m.n_cells;
    const unsigned me = cluster_rank();
    const unsigned cs = cluster_nranks();
    const int row0 = (int)me * R;
    const int nloc = max(0, min(R, C - row0));
    ff* sbuf = reinterpret_cast<ff*>(smem);                    // [3][CBS]
    float4* rb0 = reinterpret_cast<float4*>(sbuf + 3 * CBS);   // [R] (r, w, s, 1/d), buffer 0
    float4* rb1 = rb0 + R;                                     // buffer 1
    float* off = reinterpret_cast<float*>(rb1 + R);            // [W][R]
    float* diag = off + W * R;
    uint16_t* colp = reinterpret_cast<uint16_t*>(diag + R);   // [W][R] (rank << 12) | local
    const int t0 = threadIdx.x;

    for (int l = t0; l < nloc; l += CBS) {
        const int g = row0 + l;
        diag[l] = a.A.diag[g];
        bool local = true;
#pragma unroll
        for (int j = 0; j < W; ++j) {
            off[j * R + l] = a.A.off[(size_t)j * C + g];
            const int c = a.m.ell_col[(size_t)j * C + g];
            const int rk = c / R;
            colp[j * R + l] = (uint16_t)((rk << 12) | (c - rk * R));
            local = local && rk == (int)me;
        }
        local = __all_sync(__activemask(), local);
        if ((t0 & 31) == 0) chunk_local[l >> 5] = local ? 1 : 0;
    }
    // r0 = b - A x0 ; buffer 0 = (r0, 0, 0, 1/d) ; r0.r0 ; b.b
    float xr[RPT], pr[RPT], sr[RPT], rr_[RPT], ur[RPT], wr[RPT];
    ff acc[3] = {ff_zero(), ff_zero(), ff_zero()};
#pragma unroll
    for (int u = 0; u < RPT; ++u) {
        const int l = t0 + u * CBS;
        xr[u] = pr[u] = sr[u] = rr_[u] = ur[u] = wr[u] = 0.0f;
        if (l < nloc) {
            const int g = row0 + l;
            xr[u] = a.x[g];
            const float d = diag[l];
            float ax = d * xr[u];
#pragma unroll
            for (int j = 0; j < W; ++j) ax += off[j * R + l] * a.x[a.m.ell_col[(size_t)j * C + g]];
            const float bi = a.A.rhs[g];
            const float ri = bi - ax;
            rr_[u] = ri;
            rb0[l] = make_float4(ri, 0.0f, 0.0f, d != 0.0f ? 1.0f / d : 1.0f);
            ff_fma(acc[0], ri, ri);
            ff_fma(acc[2], bi, bi);
        }
    }
    unsigned parity = 0;
    ff red[3];
    cluster_reduce_tree<3>(acc, red, sbuf, slots, parity, me, cs);
    parity ^= 1u;
    if (t0 == 0) {
        const double rr0 = ff_to_double(red[0]);
        sc.thr2 = ff_norm(ff_from_double(fmax(a.atol2, a.rtol2 * rr0)));
        sc.af = 0.0f;  // pass 0 forms u0 = M r0 and w0 = A u0 and moves nothing
        sc.bf = 0.0f;
        sc.k = -1;
        sc.status = WCFD_OK;
        sc.go = 1;
        if (me == 0) {
            a.stats->initial_residual = sqrt(rr0);
            a.stats->rhs_norm = sqrt(ff_to_double(red[2]));
        }
    }
    __syncthreads();  // the cluster barrier above also published buffer 0 to every CTA
    int cur = 0;
    while (sc.go) {
        const float af = sc.af, bf = sc.bf;
        const float4* rbo = cur ? rb1 : rb0;
        float4* rbn = cur ? rb0 : rb1;
        ff acc3[3] = {ff_zero(), ff_zero(), ff_zero()};
#pragma unroll
        for (int u = 0; u < RPT; ++u) {
            const int l = t0 + u * CBS;
            if (l < nloc) {
                const float4 own = rbo[l];
                // s = w + beta s ; p = u + beta p ; x += alpha p ; r -= alpha s ; u = M r
                const float si = wr[u] + bf * sr[u];
                const float pi = ur[u] + bf * pr[u];
                xr[u] += af * pi;
                const float ri = rr_[u] - af * si;
                const float ui = ri * own.w;
                // w = A u, the neighbours' u formed from their previous (r, w, s)
                float wi = diag[l] * ui;
                if (chunk_local[l >> 5]) {  // warp-uniform: every neighbour in this CTA
#pragma unroll
                    for (int j = 0; j < W; ++j) {
                        const float4 v = rbo[colp[j * R + l] & 0xFFFu];
                        wi += off[j * R + l] * ((v.x - af * (v.y + bf * v.z)) * v.w);
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < W; ++j) {
                        const unsigned cp = colp[j * R + l];
                        const unsigned rk = cp >> 12;
                        const unsigned lo = cp & 0xFFFu;
                        const float4 v = rk == me ? rbo[lo] : ld_cluster_f32x4(map_rank(rbo + lo, rk));
                        const float uc = (v.x - af * (v.y + bf * v.z)) * v.w;
                        wi += off[j * R + l] * uc;
                    }
                }
                rbn[l] = make_float4(ri, wi, si, own.w);
                sr[u] = si;
                pr[u] = pi;
                rr_[u] = ri;
                ur[u] = ui;
                wr[u] = wi;
                ff_fma(acc3[0], ri, ri);
                ff_fma(acc3[1], ri, ui);
                ff_fma(acc3[2], wi, ui);
            }
        }
        ff d3[3];
        cluster_reduce_tree<3>(acc3, d3, sbuf, slots, parity, me, cs);
        parity ^= 1u;
        if (t0 == 0) {
            const ff rr = ff_norm(d3[0]), gamma = ff_norm(d3[1]), delta = ff_norm(d3[2]);
            sc.rr = rr;
            sc.k += 1;  // x now holds k updates
            if (!(sc.k < a.maxiter && ff_gt(rr, sc.thr2))) {
                sc.go = 0;
            } else {
                float bf_n = 0.0f;
                ff den = delta;  // p.A p
                if (sc.k > 0) {
                    bf_n = sc.gamma.hi != 0.0f ? ff_div_to_float(gamma, sc.gamma) : 0.0f;
                    // delta - beta gamma / alpha_prev, with beta and alpha_prev as used by the vectors
                    const ff corr = ff_div(ff_mul(ff{bf_n, 0.0f}, gamma), ff{sc.alpha_prev, 0.0f});
                    const ff t = ff_two_sum(den.hi, -corr.hi);
                    den = ff_norm(ff{t.hi, __fadd_rn(t.lo, __fsub_rn(den.lo, corr.lo))});
                }
                if (den.hi == 0.0f || gamma.hi == 0.0f) {
                    sc.status = WCFD_KRYLOV_BREAKDOWN;
                    sc.go = 0;
                } else {
                    sc.af = ff_div_to_float(gamma, den);
                    sc.bf = bf_n;
                    sc.alpha_prev = sc.af;
                    sc.gamma = gamma;
                }
            }
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
        a.stats->iterations = sc.k < 0 ? 0 : sc.k;
        a.stats->status = st;
        a.stats->residual = sqrt(ff_to_double(sc.rr));
    }
}

template <int W, int RPT>
__global__ void __launch_bounds__(CBS) cg1_cluster_kernel(KrylovArgs a, int R) {
    cg1_cluster_body<W, RPT>(a, R);
}

const void* cg1_cluster_kernel_for(int W, int R) {
    const int rpt = R <= CBS ? 1 : (R <= 2 * CBS ? 2 : 0);
    switch (W * 8 + rpt) {
        case 0 * 8 + 1: return (const void*)cg1_cluster_kernel<0, 1>;
        case 0 * 8 + 2: return (const void*)cg1_cluster_kernel<0, 2>;
        case 1 * 8 + 1: return (const void*)cg1_cluster_kernel<1, 1>;
        case 1 * 8 + 2: return (const void*)cg1_cluster_kernel<1, 2>;
        case 2 * 8 + 1: return (const void*)cg1_cluster_kernel<2, 1>;
        case 2 * 8 + 2: return (const void*)cg1_cluster_kernel<2, 2>;
        case 3 * 8 + 1: return (const void*)cg1_cluster_kernel<3, 1>;
        case 3 * 8 + 2: return (const void*)cg1_cluster_kernel<3, 2>;
        case 4 * 8 + 1: return (const void*)cg1_cluster_kernel<4, 1>;
        case 4 * 8 + 2: return (const void*)cg1_cluster_kernel<4, 2>;
        case 5 * 8 + 1: return (const void*)cg1_cluster_kernel<5, 1>;
        case 5 * 8 + 2: return (const void*)cg1_cluster_kernel<5, 2>;
        case 6 * 8 + 1: return (const void*)cg1_cluster_kernel<6, 1>;
        case 6 * 8 + 2: return (const void*)cg1_cluster_kernel<6, 2>;
        default: return nullptr;
    }
}

// ---------------------------------------------------------------------------------
// The single-reduction CG for the batched form, up to 4,096 rows per CTA (RPT <= 4).
//
// The (r, w, s, 1/d) double buffer above takes 32 bytes of shared memory per row, too many
// for the 4,096 rows per CTA of the batched form's largest cases.  Here only u = M r lives
// in shared memory (a single buffer), and an iteration is two phases:
//   (1) s = w + beta s ; p = u + beta p ; x += alpha p ; r -= alpha s ; u = M r, for the own
//       rows (registers, and u into shared memory), then a cluster barrier (release /
//       acquire) so that every CTA's new u is visible;
//   (2) w = A u (the neighbours' u from shared memory, DSMEM for another CTA's rows) and
//       r.r, r.u, w.u, in ONE cluster all-reduce.
// The barrier inside the all-reduce also keeps phase (1) of the next iteration from
// overwriting a u that another CTA still gathers.  Per iteration that is one plain cluster
// barrier and one all-reduce instead of the two all-reduces of textbook CG.  The values are
// those of cg1_cluster_body (the same operations per row); the scalar recurrences and the
// stop test are its own.
// Shared memory: the reduction tree, then per row u (4), off-diagonals (4 W), diag and 1/diag
// (8) and the 16-bit packed columns (2 W).
size_t cluster_cg1m_smem_bytes(int R, int W) {
    return 3 * (size_t)CBS * sizeof(ff) + (size_t)R * (6 * (size_t)W + 12);
}

template <int W, int RPT>
__device__ __forceinline__ void cg1m_cluster_body(const KrylovArgs& a, int R) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ ff slots[2 * 3 * 16];
    __shared__ unsigned char chunk_local[4096 / 32];  // 32-row chunk with no off-CTA neighbour
    struct Scal {
        ff rr, gamma, thr2;
        float af, bf, alpha_prev;
        int go, status, k;
    };
    __shared__ Scal sc;
    const int C = a.m.n_cells;
    const unsigned me = cluster_rank();
    const unsigned cs = cluster_nranks();
    const int row0 = (int)me * R;
    const int nloc = max(0, min(R, C - row0));
    ff* sbuf = reinterpret_cast<ff*>(smem);                 // [3][CBS]
    float* ub = reinterpret_cast<float*>(sbuf + 3 * CBS);   // [R] u = M r
    float* off = ub + R;                                    // [W][R]
    float* diag = off + W * R;
    float* invd = diag + R;
    uint16_t* colp = reinterpret_cast<uint16_t*>(invd + R);  // [W][R] (rank << 12) | local
    const int t0 = threadIdx.x;

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
        local = __all_sync(__activemask(), local);
        if ((t0 & 31) == 0) chunk_local[l >> 5] = local ? 1 : 0;
    }
    // r0 = b - A x0 ; u0 = M r0 ; r0.r0 ; b.b
    float xr[RPT], pr[RPT], sr[RPT], rr_[RPT], wr[RPT];
    ff acc[3] = {ff_zero(), ff_zero(), ff_zero()};
#pragma unroll
    for (int u = 0; u < RPT; ++u) {
        const int l = t0 + u * CBS;
        xr[u] = pr[u] = sr[u] = rr_[u] = wr[u] = 0.0f;
        if (l < nloc) {
            const int g = row0 + l;
            xr[u] = a.x[g];
            float ax = diag[l] * xr[u];
#pragma unroll
            for (int j = 0; j < W; ++j) ax += off[j * R + l] * a.x[a.m.ell_col[(size_t)j * C + g]];
            const float bi = a.A.rhs[g];
            const float ri = bi - ax;
            rr_[u] = ri;
            ub[l] = ri * invd[l];
            ff_fma(acc[0], ri, ri);
            ff_fma(acc[2], bi, bi);
        }
    }
    unsigned parity = 0;
    ff red[3];
    cluster_reduce_tree<3>(acc, red, sbuf, slots, parity, me, cs);
    parity ^= 1u;
    if (t0 == 0) {
        const double rr0 = ff_to_double(red[0]);
        sc.thr2 = ff_norm(ff_from_double(fmax(a.atol2, a.rtol2 * rr0)));
        sc.af = 0.0f;  // pass 0 forms w0 = A u0 and moves nothing
        sc.bf = 0.0f;
        sc.alpha_prev = 0.0f;
        sc.k = -1;
        sc.status = WCFD_OK;
        sc.go = 1;
        if (me == 0) {
            a.stats->initial_residual = sqrt(rr0);
            a.stats->rhs_norm = sqrt(ff_to_double(red[2]));
        }
    }
    __syncthreads();  // the cluster barrier above also published u0 to every CTA
    while (sc.go) {
        const float af = sc.af, bf = sc.bf;
        // (1) s = w + beta s ; p = u + beta p ; x += alpha p ; r -= alpha s ; u = M r
        if (sc.k >= 0) {
#pragma unroll
            for (int u = 0; u < RPT; ++u) {
                const int l = t0 + u * CBS;
                if (l < nloc) {
                    const float si = wr[u] + bf * sr[u];
                    const float pi = ub[l] + bf * pr[u];
                    xr[u] += af * pi;
                    const float ri = rr_[u] - af * si;
                    sr[u] = si;
                    pr[u] = pi;
                    rr_[u] = ri;
                    ub[l] = ri * invd[l];
                }
            }
            cluster_sync_all();  // every CTA's new u, visible to the cluster
        }
        // (2) w = A u ; r.r ; r.u ; w.u
        ff acc3[3] = {ff_zero(), ff_zero(), ff_zero()};
#pragma unroll
        for (int u = 0; u < RPT; ++u) {
            const int l = t0 + u * CBS;
            if (l < nloc) {
                const float ui = ub[l];
                float wi = diag[l] * ui;
                if (chunk_local[l >> 5]) {  // warp-uniform: every neighbour in this CTA
#pragma unroll
                    for (int j = 0; j < W; ++j) wi += off[j * R + l] * ub[colp[j * R + l] & 0xFFFu];
                } else {
#pragma unroll
                    for (int j = 0; j < W; ++j) {
                        const unsigned cp = colp[j * R + l];
                        const unsigned rk = cp >> 12;
                        const unsigned lo = cp & 0xFFFu;
                        const float uc = rk == me ? ub[lo] : ld_cluster_f32(map_rank(ub + lo, rk));
                        wi += off[j * R + l] * uc;
                    }
                }
                wr[u] = wi;
                const float ri = rr_[u];
                ff_fma(acc3[0], ri, ri);
                ff_fma(acc3[1], ri, ui);
                ff_fma(acc3[2], wi, ui);
            }
        }
        ff d3[3];
        cluster_reduce_tree<3>(acc3, d3, sbuf, slots, parity, me, cs);
        parity ^= 1u;
        if (t0 == 0) {
            const ff rr = ff_norm(d3[0]), gamma = ff_norm(d3[1]), delta = ff_norm(d3[2]);
            sc.rr = rr;
            sc.k += 1;  // x now holds k updates
            if (!(sc.k < a.maxiter && ff_gt(rr, sc.thr2))) {
                sc.go = 0;
            } else {
                float bf_n = 0.0f;
                ff den = delta;  // p.A p
                if (sc.k > 0) {
                    bf_n = sc.gamma.hi != 0.0f ? ff_div_to_float(gamma, sc.gamma) : 0.0f;
                    const ff corr = ff_div(ff_mul(ff{bf_n, 0.0f}, gamma), ff{sc.alpha_prev, 0.0f});
                    const ff t = ff_two_sum(den.hi, -corr.hi);
                    den = ff_norm(ff{t.hi, __fadd_rn(t.lo, __fsub_rn(den.lo, corr.lo))});
                }
                if (den.hi == 0.0f || gamma.hi == 0.0f) {
                    sc.status = WCFD_KRYLOV_BREAKDOWN;
                    sc.go = 0;
                } else {
                    sc.af = ff_div_to_float(gamma, den);
                    sc.bf = bf_n;
                    sc.alpha_prev = sc.af;
                    sc.gamma = gamma;
                }
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < RPT; ++u) {
        const int l = t0 + u * CBS;
        if (l < nloc) a.x[row0 + l] = xr[u];
    }
    if (me == 0 && t0 == 0) {
        int st = sc.status;
        if (st == WCFD_OK && !ff_le(sc.rr, sc.thr2)) st = WCFD_NOT_CONVERGED;
        a.stats->iterations = sc.k < 0 ? 0 : sc.k;
        a.stats->status = st;
        a.stats->residual = sqrt(ff_to_double(sc.rr));
    }
}

// One cluster per case of a device case table, as cg_cluster_batched (krylov_cluster.cu):
// the same systems, warm starts, refinement mode and stats, the single-reduction CG.
template <int W, int RPT>
__global__ void __launch_bounds__(CBS) cg1m_cluster_batched(const wcfd_case* __restrict__ cases, int cs, int refine) {
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
    cg1m_cluster_body<W, RPT>(a, (c.mesh.n_cells + cs - 1) / cs);
}

#define WCFD_CG1M_CASE(Wv)                                                      \
    case Wv * 8 + 1: return (const void*)cg1m_cluster_batched<Wv, 1>;           \
    case Wv * 8 + 2: return (const void*)cg1m_cluster_batched<Wv, 2>;           \
    case Wv * 8 + 4: return (const void*)cg1m_cluster_batched<Wv, 4>;

const void* cg1m_cluster_batched_for(int W, int R) {
    if (R > 4096) return nullptr;  // 12-bit local index of the packed columns
    const int rpt = cluster_cg_rpt(R);
    switch (W * 8 + rpt) {
        WCFD_CG1M_CASE(0)
        WCFD_CG1M_CASE(1)
        WCFD_CG1M_CASE(2)
        WCFD_CG1M_CASE(3)
        WCFD_CG1M_CASE(4)
        WCFD_CG1M_CASE(5)
        WCFD_CG1M_CASE(6)
        default: return nullptr;
    }
}
#undef WCFD_CG1M_CASE

}  // namespace wcfd
