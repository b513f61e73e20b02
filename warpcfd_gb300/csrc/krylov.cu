// Persistent Krylov solvers: one cooperative launch per solve, rows distributed
// grid-stride over all co-resident blocks, fp64 dot products reduced deterministically
// at bounded grid barriers (common.cuh).  They replace warp.optim.linear.cg / bicgstab
// with the diagonal (Jacobi) preconditioner as called by Equation.solve_Axb
// (warp_cfd/FV/terms/equation.py:195-200).  Stop test: ||r||_2 <= atol before an
// iteration, or maxiter iterations.
#include "common.cuh"
#include "kernels.cuh"

namespace wcfd {

constexpr int BS = kSolverBlock;

// sum_j A_ij (w_j x_j) for the NC components of row i; w = nullptr means w = 1.
template <int NC>
__device__ __forceinline__ void row_apply(const KrylovArgs& a, int i, const float* __restrict__ x,
                                          const float* __restrict__ w, float (&out)[NC]) {
    const int C = a.m.n_cells;
#pragma unroll
    for (int o = 0; o < NC; ++o) {
        const size_t q = NC * (size_t)i + o;
        const float xi = w ? x[q] * w[q] : x[q];
        out[o] = a.A.diag[q] * xi;
    }
    for (int j = 0; j < a.m.ell_width; ++j) {
        const float v = a.A.off[(size_t)j * C + i];
        const int col = __ldg(a.m.ell_col + (size_t)j * C + i);
#pragma unroll
        for (int o = 0; o < NC; ++o) {
            const size_t q = NC * (size_t)col + o;
            const float xj = w ? x[q] * w[q] : x[q];
            out[o] += v * xj;
        }
    }
}

__device__ __forceinline__ float jacobi(float d) { return d != 0.0f ? 1.0f / d : 1.0f; }

// On a failed barrier (timeout, or another block's error) every block leaves; block 0
// records the error word so the caller sees why the solve stopped.
__device__ void fail_stats(const KrylovArgs& a, int k) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.stats->iterations = k;
        a.stats->status = *((volatile int*)a.g.err);
        a.stats->residual = -1.0;
    }
}

#define SYNC(NV, arr)                                   \
    do {                                                \
        if (!grid_sync<NV, BS>(a.g, arr)) {             \
            fail_stats(a, k);                           \
            return;                                     \
        }                                               \
    } while (0)

__device__ void write_stats(const KrylovArgs& a, int k, double rr, int status) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        int st = status;
        if (st == WCFD_OK && !(rr <= a.atol2)) st = WCFD_NOT_CONVERGED;
        a.stats->iterations = k;
        a.stats->status = st;
        a.stats->residual = sqrt(rr);
    }
}

// Jacobi-preconditioned CG (scalar system).  Workspace: r, p, q, invd (4 C floats).
__global__ void __launch_bounds__(BS) cg_kernel(KrylovArgs a) {
    const int C = a.m.n_cells;
    float* r = a.ws;
    float* p = a.ws + (size_t)C;
    float* q = a.ws + 2 * (size_t)C;
    float* invd = a.ws + 3 * (size_t)C;
    const float* b = a.A.rhs;
    float* x = a.x;
    const int stride = gridDim.x * BS;
    const int i0 = blockIdx.x * BS + threadIdx.x;

    // r = b - A x ; z = M r ; p = z ; rr = r.r ; rz = r.z
    double red[2] = {0.0, 0.0};
    for (int i = i0; i < C; i += stride) {
        float ax[1];
        row_apply<1>(a, i, x, nullptr, ax);
        const float ri = b[i] - ax[0];
        const float di = jacobi(a.A.diag[i]);
        const float zi = ri * di;
        r[i] = ri;
        invd[i] = di;
        p[i] = zi;
        red[0] += (double)ri * ri;
        red[1] += (double)ri * zi;
    }
    int k = 0, status = WCFD_OK;
    SYNC(2, red);
    double rr = red[0], rz = red[1];
    while (k < a.maxiter && rr > a.atol2) {
        double pq[1] = {0.0};
        for (int i = i0; i < C; i += stride) {
            float qi[1];
            row_apply<1>(a, i, p, nullptr, qi);
            q[i] = qi[0];
            pq[0] += (double)p[i] * qi[0];
        }
        SYNC(1, pq);
        if (pq[0] == 0.0) { status = WCFD_KRYLOV_BREAKDOWN; break; }
        const double alpha = rz / pq[0];
        const float af = (float)alpha;
        double red2[2] = {0.0, 0.0};
        for (int i = i0; i < C; i += stride) {
            x[i] += af * p[i];
            const float ri = r[i] - af * q[i];
            r[i] = ri;
            const float zi = ri * invd[i];
            red2[0] += (double)ri * ri;
            red2[1] += (double)ri * zi;
        }
        SYNC(2, red2);
        rr = red2[0];
        const double beta = rz != 0.0 ? red2[1] / rz : 0.0;
        rz = red2[1];
        const float bf = (float)beta;
        for (int i = i0; i < C; i += stride) p[i] = r[i] * invd[i] + bf * p[i];
        SYNC(0, nullptr);
        ++k;
    }
    write_stats(a, k, rr, status);
}

// Right-preconditioned (Jacobi) BiCGSTAB on the 3-component momentum system.
// Workspace: r, r0, p, v, t, invd (6 x 3C floats).  s overwrites r.
__global__ void __launch_bounds__(BS) bicgstab_kernel(KrylovArgs a) {
    const int C = a.m.n_cells;
    const size_t n3 = 3 * (size_t)C;
    float* r = a.ws;
    float* r0 = a.ws + n3;
    float* p = a.ws + 2 * n3;
    float* v = a.ws + 3 * n3;
    float* t = a.ws + 4 * n3;
    float* invd = a.ws + 5 * n3;
    const float* b = a.A.rhs;
    float* x = a.x;
    const int stride = gridDim.x * BS;
    const int i0 = blockIdx.x * BS + threadIdx.x;

    double red[2] = {0.0, 0.0};
    for (int i = i0; i < C; i += stride) {
        float ax[3];
        row_apply<3>(a, i, x, nullptr, ax);
#pragma unroll
        for (int o = 0; o < 3; ++o) {
            const size_t q = 3 * (size_t)i + o;
            const float ri = b[q] - ax[o];
            r[q] = ri;
            r0[q] = ri;
            p[q] = ri;
            invd[q] = jacobi(a.A.diag[q]);
            red[0] += (double)ri * ri;
        }
    }
    int k = 0, status = WCFD_OK;
    SYNC(1, red);
    double rr = red[0];
    double rho = rr;
    while (k < a.maxiter && rr > a.atol2) {
        // v = A (M p) ; r0.v
        double r0v[1] = {0.0};
        for (int i = i0; i < C; i += stride) {
            float vi[3];
            row_apply<3>(a, i, p, invd, vi);
#pragma unroll
            for (int o = 0; o < 3; ++o) {
                const size_t q = 3 * (size_t)i + o;
                v[q] = vi[o];
                r0v[0] += (double)r0[q] * vi[o];
            }
        }
        SYNC(1, r0v);
        if (r0v[0] == 0.0) { status = WCFD_KRYLOV_BREAKDOWN; break; }
        const double alpha = rho / r0v[0];
        const float af = (float)alpha;
        // s = r - alpha v (in r) ; x += alpha M p
        for (int i = i0; i < C; i += stride) {
#pragma unroll
            for (int o = 0; o < 3; ++o) {
                const size_t q = 3 * (size_t)i + o;
                r[q] = r[q] - af * v[q];
                x[q] += af * (p[q] * invd[q]);
            }
        }
        SYNC(0, nullptr);
        // t = A (M s) ; t.t ; t.s
        double ts[2] = {0.0, 0.0};
        for (int i = i0; i < C; i += stride) {
            float ti[3];
            row_apply<3>(a, i, r, invd, ti);
#pragma unroll
            for (int o = 0; o < 3; ++o) {
                const size_t q = 3 * (size_t)i + o;
                t[q] = ti[o];
                ts[0] += (double)ti[o] * ti[o];
                ts[1] += (double)ti[o] * r[q];
            }
        }
        SYNC(2, ts);
        const double omega = ts[0] != 0.0 ? ts[1] / ts[0] : 0.0;
        const float of = (float)omega;
        // x += omega M s ; r = s - omega t ; r.r ; r0.r
        double rr2[2] = {0.0, 0.0};
        for (int i = i0; i < C; i += stride) {
#pragma unroll
            for (int o = 0; o < 3; ++o) {
                const size_t q = 3 * (size_t)i + o;
                const float si = r[q];
                x[q] += of * (si * invd[q]);
                const float ri = si - of * t[q];
                r[q] = ri;
                rr2[0] += (double)ri * ri;
                rr2[1] += (double)r0[q] * ri;
            }
        }
        SYNC(2, rr2);
        rr = rr2[0];
        ++k;
        if (omega == 0.0 || rho == 0.0) { status = WCFD_KRYLOV_BREAKDOWN; break; }
        const double beta = (rr2[1] / rho) * (alpha / omega);
        rho = rr2[1];
        const float bf = (float)beta;
        // p = r + beta (p - omega v)
        for (int i = i0; i < C; i += stride) {
#pragma unroll
            for (int o = 0; o < 3; ++o) {
                const size_t q = 3 * (size_t)i + o;
                p[q] = r[q] + bf * (p[q] - of * v[q]);
            }
        }
        SYNC(0, nullptr);
    }
    write_stats(a, k, rr, status);
}

}  // namespace wcfd
