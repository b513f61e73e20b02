// Persistent Krylov solvers: one cooperative launch per solve, rows distributed
// grid-stride over all co-resident blocks, fp64-accurate dot products (exact products
// summed in float-float across threads, warps and blocks; common.cuh) reduced deterministically at bounded grid barriers.  They replace warp.optim.linear.cg /
// bicgstab with the diagonal (Jacobi) preconditioner as called by Equation.solve_Axb
// (warp_cfd/FV/terms/equation.py:195-200).  Stop test: ||r||_2 <= atol before an
// iteration, or maxiter iterations.
//
// Each search-direction update (CG: p = z + beta p; BiCGSTAB: p = r + beta (p - omega v),
// s = r - alpha v) is evaluated on the fly inside the SpMV that consumes it, for the row
// itself and for every gathered neighbour, and the new direction is written to the other
// half of a double buffer.  The arithmetic is the textbook algorithm's, but a CG iteration
// needs two grid barriers instead of three and a BiCGSTAB iteration three instead of five.
//
// The scalar recurrences (alpha, beta, omega, the stop test) run on the float-float sums
// in thread 0 of each block and reach the other threads through shared memory: GB300
// runs fp64 at about 1/64 of its fp32 rate (a dependent fp64 division costs about 600
// cycles), and every thread of the grid waits for these few operations.
#include "common.cuh"
#include "kernels.cuh"

namespace wcfd {

constexpr int BS = kSolverBlock;

__device__ __forceinline__ float jacobi(float d) { return d != 0.0f ? 1.0f / d : 1.0f; }

// Krylov scalars of one block, owned by thread 0
struct KScalars {
    ff rr, rz, rho, alpha, omega, thr2;
    float af, bf, of;
    int go, status, k;
};

// On a failed barrier (timeout, or another block's error) every block leaves; block 0
// records the error word so the caller sees why the solve stopped.
__device__ void fail_stats(const KrylovArgs& a, int k) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.stats->iterations = k;
        a.stats->status = *((volatile int*)a.g.err);
        a.stats->residual = -1.0;
    }
}

// block-reduce the float-float accumulators `acc` and sum them over the grid into the
// float-float array `out` (NV values)
#define SYNC(NV, acc, out)                                         \
    do {                                                           \
        block_reduce_ff<NV, BS>(acc);                              \
        if (!grid_sync<NV, BS>(a.g, acc, out, ++phase)) {          \
            fail_stats(a, sc.k);                                   \
            return;                                                \
        }                                                          \
    } while (0)

// set-up scalars from the initial r.r and b.b; block 0 records ||r_0|| and ||b||
__device__ void init_scalars(const KrylovArgs& a, KScalars& sc, const ff& rr, const ff& bb) {
    const double rr0 = ff_to_double(rr);
    sc.rr = rr;
    sc.thr2 = ff_norm(ff_from_double(fmax(a.atol2, a.rtol2 * rr0)));
    sc.go = (0 < a.maxiter && ff_gt(sc.rr, sc.thr2));
    if (blockIdx.x == 0) {
        a.stats->initial_residual = sqrt(rr0);
        a.stats->rhs_norm = sqrt(ff_to_double(bb));
    }
}

__device__ void write_stats(const KrylovArgs& a, const KScalars& sc) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        int st = sc.status;
        if (st == WCFD_OK && !ff_le(sc.rr, sc.thr2)) st = WCFD_NOT_CONVERGED;
        a.stats->iterations = sc.k;
        a.stats->status = st;
        a.stats->residual = sqrt(ff_to_double(sc.rr));
    }
}

// L2 prefetch of the matrix lines that a warp's rows use `ahead` grid-stride trips of one
// row later: lane l < 2 W takes slab l (columns, then coefficients) and prefetches the
// lines of the warp's first and last row there (one line when the 32 rows are 128-byte
// aligned).  Nothing waits on a prefetch and no register is held.  Used by the BiCGSTAB,
// whose vectors (nine 3C arrays) exceed L2 anyway, where it takes a DRAM round trip out of
// each trip of the SpMV passes (0.374 -> 0.338 ms per 128^3 momentum solve).  The grid CG
// keeps its vectors in L2 and reads the matrix evict-first; every prefetch variant tried
// there (per line at normal priority, or a bulk prefetch of each block's 4 KB slabs with
// the evict-first policy, 1 to 5 trips ahead) made its iteration slower (35.4 us ->
// 41-47 us on 128^3).
template <int W>
__device__ __forceinline__ void prefetch_matrix_lines(const int* col, const float* off, int C, int stride, int i,
                                                      int ahead) {
    if constexpr (W > 0) {
        const int lane = threadIdx.x & 31;
        if (lane < 2 * W) {
            const long long rb = (long long)i - lane + (long long)ahead * stride;
            if (rb < C) {
                const long long rl = rb + 31 < C ? rb + 31 : C - 1;
                const char* base = lane < W ? reinterpret_cast<const char*>(col + (size_t)lane * C)
                                            : reinterpret_cast<const char*>(off + (size_t)(lane - W) * C);
                asm volatile("prefetch.global.L2 [%0];" ::"l"(base + (size_t)rb * 4));
                asm volatile("prefetch.global.L2 [%0];" ::"l"(base + (size_t)rl * 4));
            }
        }
    }
}

// Column of slot j of row i: from the int16 offsets (kD, wcfd_mesh.ell_dcol) or the int32
// columns, streamed (evict-first) or with a plain load.
template <bool kD, bool kStream>
__device__ __forceinline__ int ell_column(const int* __restrict__ col, const int16_t* __restrict__ dcol, size_t idx,
                                          int i) {
    if constexpr (kD) return i + (int)(kStream ? __ldcs(dcol + idx) : dcol[idx]);
    else return kStream ? __ldcs(col + idx) : col[idx];
}

// Jacobi-preconditioned CG on a scalar system, W = off-diagonal width known at compile
// time so the loads of a row's columns and gathered values are all in flight at once.
// Workspace: r, pA, pB, q, invd, z (6 C floats).
//
// The matrix (off-diagonals and columns, 8 W bytes a row) is read with the streaming
// (evict-first) cache policy: it is re-read every iteration but does not fit L2 next to
// the vectors on large meshes, and evicting it first keeps the vectors (gathered and
// re-read within the iteration) resident in the 129 MB L2.
//
// Per iteration: (1) p_new = z + beta p_old for the row and every neighbour, q = A p_new,
// p.q -- and x += alpha_prev p_old, the previous iteration's solution update, which reads
// the p_old this pass loads anyway; (2) r -= alpha q, z = r / diag, r.r and r.z.  Each
// thread takes two rows (i, i + stride) per trip of pass (1) so that twice the column,
// coefficient and gather loads are in flight: the pass is bound by memory latency, not
// by bandwidth, at one row per thread.
//
// kD: the columns come from the int16 offsets (wcfd_mesh.ell_dcol) instead of the int32
// columns, 6 W instead of 8 W streamed bytes per row (the same columns, the same bits):
// pass (1) streams the matrix from DRAM while the vectors stay in L2, so on the 128^3
// cavity (W = 6) an iteration went from 35.5 to 33.3 us.  The BiCGSTAB keeps the int32
// columns: the offsets made its solve slower there (0.338 -> 0.360 ms).
template <int W, bool kD>
__global__ void __launch_bounds__(BS, 1) cg_kernel(KrylovArgs a) {
    __shared__ KScalars sc;
    const int C = a.m.n_cells;
    float* r = a.ws;
    float* pbuf[2] = {a.ws + (size_t)C, a.ws + 2 * (size_t)C};
    float* q = a.ws + 3 * (size_t)C;
    float* invd = a.ws + 4 * (size_t)C;
    float* z = a.ws + 5 * (size_t)C;
    const float* __restrict__ b = a.A.rhs;
    const float* __restrict__ diag = a.A.diag;
    const float* __restrict__ off = a.A.off;
    const int* __restrict__ col = a.m.ell_col;
    const int16_t* __restrict__ dcol = a.m.ell_dcol;
    float* x = a.x;
    const int stride = gridDim.x * BS;
    const int i0 = blockIdx.x * BS + threadIdx.x;
    unsigned phase = 0;
    if (threadIdx.x == 0) {
        sc.k = 0;
        sc.status = WCFD_OK;
    }

    // r = b - A x ; z = M r ; p = z ; rr = r.r ; rz = r.z ; bb = b.b
    ff acc[3] = {ff_zero(), ff_zero(), ff_zero()};
    for (int i = i0; i < C; i += stride) {
        float ax = diag[i] * x[i];
#pragma unroll
        for (int j = 0; j < W; ++j) ax += off[(size_t)j * C + i] * x[ell_column<kD, false>(col, dcol, (size_t)j * C + i, i)];
        const float ri = b[i] - ax;
        const float di = jacobi(diag[i]);
        const float zi = ri * di;
        r[i] = ri;
        invd[i] = di;
        z[i] = zi;
        pbuf[0][i] = zi;
        ff_fma(acc[0], ri, ri);
        ff_fma(acc[1], ri, zi);
        ff_fma(acc[2], b[i], b[i]);
    }
    ff red[3];
    SYNC(3, acc, red);
    if (threadIdx.x == 0) {
        init_scalars(a, sc, red[0], red[2]);
        sc.rz = red[1];
        sc.bf = 0.0f;  // the first direction is z itself
        sc.af = 0.0f;
    }
    __syncthreads();
    int cur = 0;
    float pending = 0.0f;  // alpha of the last completed iteration, not yet added to x
    while (sc.go) {
        const float bf = sc.bf;
        const float ap = pending;
        const float* po = pbuf[cur];  // written by other blocks in this launch: no restrict
        float* pn = pbuf[cur ^ 1];
        // x += alpha_prev p_old ; p_new = z + beta p_old (row and neighbours) ; q = A p_new ; p.q
        ff accq[1] = {ff_zero()};
        for (int i = i0; i < C; i += 2 * stride) {
            const int i2 = i + stride;
            const bool two = i2 < C;
            const int k2 = two ? i2 : i;  // a lone last row loads itself twice, stores once
            constexpr int WA = W > 0 ? W : 1;  // no zero-length arrays for W = 0
            int c1[WA], c2[WA];
            float o1[WA], o2[WA];
#pragma unroll
            for (int j = 0; j < W; ++j) {
                c1[j] = ell_column<kD, true>(col, dcol, (size_t)j * C + i, i);
                c2[j] = ell_column<kD, true>(col, dcol, (size_t)j * C + k2, k2);
            }
#pragma unroll
            for (int j = 0; j < W; ++j) {
                o1[j] = __ldcs(off + (size_t)j * C + i);
                o2[j] = __ldcs(off + (size_t)j * C + k2);
            }
            const float po1 = po[i], po2 = po[k2];
            const float p1 = z[i] + bf * po1;
            const float p2 = z[k2] + bf * po2;
            float q1 = diag[i] * p1;
            float q2 = diag[k2] * p2;
            float g1[WA], g2[WA];
#pragma unroll
            for (int j = 0; j < W; ++j) {
                g1[j] = z[c1[j]] + bf * po[c1[j]];
                g2[j] = z[c2[j]] + bf * po[c2[j]];
            }
#pragma unroll
            for (int j = 0; j < W; ++j) {
                q1 += o1[j] * g1[j];
                q2 += o2[j] * g2[j];
            }
            if (ap != 0.0f) x[i] += ap * po1;
            pn[i] = p1;
            q[i] = q1;
            ff_fma(accq[0], p1, q1);
            if (two) {
                if (ap != 0.0f) x[i2] += ap * po2;
                pn[i2] = p2;
                q[i2] = q2;
                ff_fma(accq[0], p2, q2);
            }
        }
        ff pq[1];
        SYNC(1, accq, pq);
        if (threadIdx.x == 0) {
            if (pq[0].hi == 0.0f) {
                sc.status = WCFD_KRYLOV_BREAKDOWN;
                sc.go = 0;
            } else {
                sc.af = ff_div_to_float(sc.rz, pq[0]);
            }
        }
        __syncthreads();
        pending = 0.0f;  // alpha_prev p_old is in x now
        if (!sc.go) break;
        const float af = sc.af;
        // r -= alpha q ; z = M r ; rr ; rz
        ff acc2[2] = {ff_zero(), ff_zero()};
        for (int i = i0; i < C; i += stride) {
            const float ri = r[i] - af * q[i];
            r[i] = ri;
            const float zi = ri * invd[i];
            z[i] = zi;
            ff_fma(acc2[0], ri, ri);
            ff_fma(acc2[1], ri, zi);
        }
        ff red2[2];
        SYNC(2, acc2, red2);
        if (threadIdx.x == 0) {
            sc.rr = red2[0];
            sc.bf = sc.rz.hi != 0.0f ? ff_div_to_float(red2[1], sc.rz) : 0.0f;
            sc.rz = red2[1];
            sc.k += 1;
            sc.go = (sc.k < a.maxiter && ff_gt(sc.rr, sc.thr2));
        }
        __syncthreads();
        pending = af;
        cur ^= 1;
    }
    // the last iteration's x += alpha p (its p is pbuf[cur] after the swap)
    if (pending != 0.0f) {
        const float* pl = pbuf[cur];
        for (int i = i0; i < C; i += stride) x[i] += pending * pl[i];
    }
    write_stats(a, sc);
}

// Right-preconditioned (Jacobi) BiCGSTAB on the 3-component momentum system
// (interleaved rows 3c+o, shared off-diagonals).
// Workspace (3C floats each): r, r0, pA, pB, vA, vB, t, s, invd.
template <int W>
__global__ void __launch_bounds__(BS) bicgstab_kernel(KrylovArgs a) {
    __shared__ KScalars sc;
    const int C = a.m.n_cells;
    const size_t n3 = 3 * (size_t)C;
    float* r = a.ws;
    float* r0 = a.ws + n3;
    float* pbuf[2] = {a.ws + 2 * n3, a.ws + 3 * n3};
    float* vbuf[2] = {a.ws + 4 * n3, a.ws + 5 * n3};
    float* t = a.ws + 6 * n3;
    float* s = a.ws + 7 * n3;
    float* invd = a.ws + 8 * n3;
    const float* __restrict__ b = a.A.rhs;
    const float* __restrict__ diag = a.A.diag;
    const float* __restrict__ off = a.A.off;
    const int* __restrict__ col = a.m.ell_col;
    float* x = a.x;
    const int stride = gridDim.x * BS;
    const int i0 = blockIdx.x * BS + threadIdx.x;
    unsigned phase = 0;
    if (threadIdx.x == 0) {
        sc.k = 0;
        sc.status = WCFD_OK;
    }

    // r = b - A x ; r0 = r ; p = r ; v = 0 ; rr ; rho = r0.r = rr ; bb = b.b
    ff acc[2] = {ff_zero(), ff_zero()};
    for (int i = i0; i < C; i += stride) {
        float ax[3];
#pragma unroll
        for (int o = 0; o < 3; ++o) ax[o] = diag[3 * (size_t)i + o] * x[3 * (size_t)i + o];
#pragma unroll
        for (int j = 0; j < W; ++j) {
            const float v = __ldcs(off + (size_t)j * C + i);
            const int c = __ldcs(col + (size_t)j * C + i);
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
            invd[q] = jacobi(diag[q]);
            ff_fma(acc[0], ri, ri);
            ff_fma(acc[1], b[q], b[q]);
        }
    }
    ff red[2];
    SYNC(2, acc, red);
    if (threadIdx.x == 0) {
        init_scalars(a, sc, red[0], red[1]);
        sc.rho = red[0];
        sc.bf = 0.0f;  // the first direction is r itself
        sc.of = 0.0f;
    }
    __syncthreads();
    int cur = 0;
    while (sc.go) {
        const float bf = sc.bf, of0 = sc.of;
        const float* po = pbuf[cur];  // written by other blocks in this launch: no restrict
        const float* vo = vbuf[cur];
        float* pn = pbuf[cur ^ 1];
        float* vn = vbuf[cur ^ 1];
        // p = r + beta (p - omega v) ; v = A (M p) ; r0.v
        ff accv[1] = {ff_zero()};
        for (int i = i0; i < C; i += stride) {
            prefetch_matrix_lines<W>(col, off, C, stride, i, 1);
            float pi[3], vi[3];
#pragma unroll
            for (int o = 0; o < 3; ++o) {
                const size_t q = 3 * (size_t)i + o;
                pi[o] = r[q] + bf * (po[q] - of0 * vo[q]);
                vi[o] = diag[q] * (pi[o] * invd[q]);
            }
#pragma unroll
            for (int j = 0; j < W; ++j) {
                const float v = __ldcs(off + (size_t)j * C + i);
                const int c = __ldcs(col + (size_t)j * C + i);
#pragma unroll
                for (int o = 0; o < 3; ++o) {
                    const size_t q = 3 * (size_t)c + o;
                    const float pc = r[q] + bf * (po[q] - of0 * vo[q]);
                    vi[o] += v * (pc * invd[q]);
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
        SYNC(1, accv, r0v);
        if (threadIdx.x == 0) {
            if (r0v[0].hi == 0.0f) {
                sc.status = WCFD_KRYLOV_BREAKDOWN;
                sc.go = 0;
            } else {
                sc.alpha = ff_div(sc.rho, r0v[0]);
                sc.af = ff_to_float(sc.alpha);
            }
        }
        __syncthreads();
        if (!sc.go) break;
        const float af = sc.af;
        // s = r - alpha v ; x += alpha M p ; t = A (M s) ; t.t ; t.s
        ff acct[2] = {ff_zero(), ff_zero()};
        for (int i = i0; i < C; i += stride) {
            prefetch_matrix_lines<W>(col, off, C, stride, i, 1);
            float si[3], ti[3];
#pragma unroll
            for (int o = 0; o < 3; ++o) {
                const size_t q = 3 * (size_t)i + o;
                si[o] = r[q] - af * vn[q];
                x[q] += af * (pn[q] * invd[q]);
                ti[o] = diag[q] * (si[o] * invd[q]);
            }
#pragma unroll
            for (int j = 0; j < W; ++j) {
                const float v = __ldcs(off + (size_t)j * C + i);
                const int c = __ldcs(col + (size_t)j * C + i);
#pragma unroll
                for (int o = 0; o < 3; ++o) {
                    const size_t q = 3 * (size_t)c + o;
                    const float scv = r[q] - af * vn[q];
                    ti[o] += v * (scv * invd[q]);
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
        SYNC(2, acct, ts);
        if (threadIdx.x == 0) {
            sc.omega = ts[0].hi != 0.0f ? ff_div(ts[1], ts[0]) : ff_zero();
            sc.of = ff_to_float(sc.omega);
        }
        __syncthreads();
        const float of = sc.of;
        // x += omega M s ; r = s - omega t ; r.r ; r0.r -- every load of the row issued
        // before its first store (x and r may alias the others as far as the compiler
        // knows), components accumulated in order
        ff accr[2] = {ff_zero(), ff_zero()};
        for (int i = i0; i < C; i += stride) {
            float sv[3], dv[3], xv[3], tv[3], rv0[3];
#pragma unroll
            for (int o = 0; o < 3; ++o) {
                const size_t q = 3 * (size_t)i + o;
                sv[o] = s[q];
                dv[o] = invd[q];
                xv[o] = x[q];
                tv[o] = t[q];
                rv0[o] = r0[q];
            }
#pragma unroll
            for (int o = 0; o < 3; ++o) {
                const size_t q = 3 * (size_t)i + o;
                x[q] = xv[o] + of * (sv[o] * dv[o]);
                const float ri = sv[o] - of * tv[o];
                r[q] = ri;
                ff_fma(accr[0], ri, ri);
                ff_fma(accr[1], rv0[o], ri);
            }
        }
        ff rr2[2];
        SYNC(2, accr, rr2);
        if (threadIdx.x == 0) {
            sc.rr = rr2[0];
            sc.k += 1;
            if (sc.omega.hi == 0.0f || sc.rho.hi == 0.0f) {
                sc.status = WCFD_KRYLOV_BREAKDOWN;
                sc.go = 0;
            } else {
                sc.bf = ff_to_float(ff_mul(ff_div(rr2[1], sc.rho), ff_div(sc.alpha, sc.omega)));
                sc.rho = rr2[1];
                sc.go = (sc.k < a.maxiter && ff_gt(sc.rr, sc.thr2));
            }
        }
        __syncthreads();
        cur ^= 1;
    }
    write_stats(a, sc);
}

// ---------------------------------------------------------------------------------
// fp64 iterative refinement of a scalar solve (the precision form of the pressure solve):
// the solution is kept in fp64 and each sweep solves for a correction with the fp32 CG
// against the residual r = b - A x computed in fp64.  The few fp64 operations per row per
// sweep (not per Krylov iteration) are affordable at GB300's fp64 rate.
template <int W>
__global__ void __launch_bounds__(kBlock) residual64_kernel(wcfd_mesh m, wcfd_system A, const double* __restrict__ x,
                                                            float* __restrict__ r) {
    const int i = blockIdx.x * kBlock + threadIdx.x;
    const int C = m.n_cells;
    if (i >= C) return;
    double acc = (double)A.diag[i] * x[i];
#pragma unroll
    for (int j = 0; j < W; ++j) acc += (double)A.off[(size_t)j * C + i] * x[m.ell_col[(size_t)j * C + i]];
    r[i] = (float)((double)A.rhs[i] - acc);
}

// running total of the correction solves' iterations over the refinement sweeps; the last
// sweep writes the total into its statistics
__global__ void refine_count_kernel(wcfd_solve_stats* stats, int* acc, int first, int last) {
    const int a = (first ? 0 : *acc) + stats->iterations;
    *acc = a;
    if (last) stats->iterations = a;
}

__global__ void __launch_bounds__(kBlock) refine_update_kernel(int C, double* __restrict__ x64,
                                                               const float* __restrict__ d, float* __restrict__ x32) {
    const int i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= C) return;
    const double v = x64[i] + (double)d[i];
    x64[i] = v;
    x32[i] = (float)v;
}

const void* residual64_kernel_for(int W) {
    switch (W) {
        case 0: return (const void*)residual64_kernel<0>;
        case 1: return (const void*)residual64_kernel<1>;
        case 2: return (const void*)residual64_kernel<2>;
        case 3: return (const void*)residual64_kernel<3>;
        case 4: return (const void*)residual64_kernel<4>;
        case 5: return (const void*)residual64_kernel<5>;
        case 6: return (const void*)residual64_kernel<6>;
        default: return nullptr;
    }
}

// Self-check of the grid barrier: `phases` barriers of two sums over all blocks; every block
// checks the sums it receives against their closed form and ORs 1 into *bad on a mismatch.
// With skip >= 0 that block returns before it arrives at the first barrier, so every other
// block's wait runs out: they record WCFD_BARRIER_TIMEOUT in the error word and return (a
// failure made without a fault: nothing ever sets the count they wait for).
__global__ void __launch_bounds__(BS, 1) barrier_check_kernel(GridCtl g, int skip, int phases, int* bad) {
    if ((int)blockIdx.x == skip) return;
    unsigned phase = 0;
    const float G = (float)gridDim.x;
    for (int p = 0; p < phases; ++p) {
        ff acc[2] = {ff{(float)(blockIdx.x + 1 + p), 0.0f}, ff{1.0f, 0.0f}};
        ff out[2];
        if (threadIdx.x != 0) acc[0] = acc[1] = ff_zero();
        if (!grid_sync<2, BS>(g, acc, out, ++phase)) return;
        const float want0 = G * (G + 1.0f) * 0.5f + G * (float)p;  // exact below 2^24
        if (threadIdx.x == 0 && (ff_to_double(out[0]) != (double)want0 || ff_to_double(out[1]) != (double)G))
            atomicOr(bad, 1);
    }
}

const void* barrier_check_kernel_ptr() { return (const void*)barrier_check_kernel; }

// W = 0 has no columns to read: its offset form is the plain one
template <bool kD>
const void* cg_kernel_pick(int W) {
    switch (W) {
        case 0: return (const void*)cg_kernel<0, false>;
        case 1: return (const void*)cg_kernel<1, kD>;
        case 2: return (const void*)cg_kernel<2, kD>;
        case 3: return (const void*)cg_kernel<3, kD>;
        case 4: return (const void*)cg_kernel<4, kD>;
        case 5: return (const void*)cg_kernel<5, kD>;
        case 6: return (const void*)cg_kernel<6, kD>;
        default: return nullptr;
    }
}

const void* bicgstab_kernel_for(int W) {
    switch (W) {
        case 0: return (const void*)bicgstab_kernel<0>;
        case 1: return (const void*)bicgstab_kernel<1>;
        case 2: return (const void*)bicgstab_kernel<2>;
        case 3: return (const void*)bicgstab_kernel<3>;
        case 4: return (const void*)bicgstab_kernel<4>;
        case 5: return (const void*)bicgstab_kernel<5>;
        case 6: return (const void*)bicgstab_kernel<6>;
        default: return nullptr;
    }
}

const void* cg_kernel_for(int W, bool delta) { return delta ? cg_kernel_pick<true>(W) : cg_kernel_pick<false>(W); }

}  // namespace wcfd
