// Device convergence monitor: the residual norms of FVM.check_convergence
// (warp_cfd/FV/model.py:278-316 with the criteria of FV/Convergence.py:53-61) in one fused
// pass and one merge, so a convergence check costs two launches and one copy of nine
// doubles instead of a host round trip per norm.
//
//   out[0..2]  ||A x - b||_2 per momentum component (the momentum system of the outer
//              iteration applied to the corrected velocity, model.py:287-296)
//   out[3..5]  ||b||_2 per component (the denominators of the relative criteria)
//   out[6]     ||div||_1            (continuity and local continuity, Convergence.py:91-100)
//   out[7]     ||rUA grad p||_inf   (velocity correction, incompressible.py:152)
//   out[8]     ||p||_inf            (pressure correction: the new pressure, incompressible.py:165)
//
// Sums of squares and of absolute values are exact products accumulated in float-float
// (common.cuh), merged per block and then across blocks in block order: the same bits on
// every run.
#include "common.cuh"
#include "kernels.cuh"

namespace wcfd {

constexpr int kNormSums = 7;          // res2[3], b2[3], div1
constexpr int kNormBlocks = 1024;     // most blocks of the partial pass

__global__ void __launch_bounds__(kBlock) norms_partial_kernel(wcfd_mesh m, wcfd_system A, const float* __restrict__ x,
                                                                const float* __restrict__ div,
                                                                const float* __restrict__ grad,
                                                                const float* __restrict__ rua,
                                                                const float* __restrict__ p, float* __restrict__ part) {
    const int C = m.n_cells, W = m.ell_width;
    ff acc[kNormSums];
#pragma unroll
    for (int k = 0; k < kNormSums; ++k) acc[k] = ff_zero();
    float vmax = 0.0f, pmax = 0.0f;
    for (int i = blockIdx.x * kBlock + threadIdx.x; i < C; i += gridDim.x * kBlock) {
        float ax[3];
#pragma unroll
        for (int o = 0; o < 3; ++o) ax[o] = A.diag[3 * (size_t)i + o] * x[3 * (size_t)i + o];
        for (int j = 0; j < W; ++j) {
            const float v = A.off[(size_t)j * C + i];
            const int c = m.ell_col[(size_t)j * C + i];
#pragma unroll
            for (int o = 0; o < 3; ++o) ax[o] += v * x[3 * (size_t)c + o];
        }
#pragma unroll
        for (int o = 0; o < 3; ++o) {
            const float b = A.rhs[3 * (size_t)i + o];
            const float r = ax[o] - b;
            ff_fma(acc[o], r, r);
            ff_fma(acc[3 + o], b, b);
        }
        if (div) ff_fma(acc[6], fabsf(div[i]), 1.0f);
        if (grad && rua) {
#pragma unroll
            for (int o = 0; o < 3; ++o) vmax = fmaxf(vmax, fabsf(rua[i] * grad[12 * (size_t)i + 9 + o]));
        }
        if (p) pmax = fmaxf(pmax, fabsf(p[i]));
    }
    block_reduce_ff<kNormSums, kBlock>(acc);
    __shared__ float smax[2][kBlock / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
        pmax = fmaxf(pmax, __shfl_xor_sync(0xffffffffu, pmax, o));
    }
    if (lane == 0) {
        smax[0][wid] = vmax;
        smax[1][wid] = pmax;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float* q = part + (size_t)blockIdx.x * (2 * kNormSums + 2);
#pragma unroll
        for (int k = 0; k < kNormSums; ++k) {
            q[2 * k] = acc[k].hi;
            q[2 * k + 1] = acc[k].lo;
        }
        float a = 0.0f, b = 0.0f;
        for (int w = 0; w < kBlock / 32; ++w) {
            a = fmaxf(a, smax[0][w]);
            b = fmaxf(b, smax[1][w]);
        }
        q[2 * kNormSums] = a;
        q[2 * kNormSums + 1] = b;
    }
}

__global__ void __launch_bounds__(32) norms_final_kernel(int nb, const float* __restrict__ part, double* __restrict__ out) {
    const int lane = threadIdx.x;
    ff acc[kNormSums];
#pragma unroll
    for (int k = 0; k < kNormSums; ++k) acc[k] = ff_zero();
    float vmax = 0.0f, pmax = 0.0f;
    for (int b = lane; b < nb; b += 32) {
        const float* q = part + (size_t)b * (2 * kNormSums + 2);
#pragma unroll
        for (int k = 0; k < kNormSums; ++k) ff_merge(acc[k], ff{q[2 * k], q[2 * k + 1]});
        vmax = fmaxf(vmax, q[2 * kNormSums]);
        pmax = fmaxf(pmax, q[2 * kNormSums + 1]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < kNormSums; ++k) ff_shfl_merge(acc[k], o);
        vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
        pmax = fmaxf(pmax, __shfl_xor_sync(0xffffffffu, pmax, o));
    }
    if (lane == 0) {
        for (int k = 0; k < 6; ++k) out[k] = sqrt(ff_to_double(acc[k]));
        out[6] = ff_to_double(acc[6]);
        out[7] = vmax;
        out[8] = pmax;
    }
}

}  // namespace wcfd

using namespace wcfd;

extern "C" int64_t wcfd_convergence_scratch_floats(void) { return (int64_t)kNormBlocks * (2 * kNormSums + 2); }

extern "C" int wcfd_convergence_norms(const wcfd_mesh* m, wcfd_system A, const float* x, const float* div,
                                      const float* cell_gradients, const float* rua, const float* p, float* scratch,
                                      double* out, void* stream) {
    if (!m || !x || !out || !scratch || !A.diag || !A.off || !A.rhs || A.ncomp != 3 || m->n_cells <= 0 ||
        m->ell_width < 0 || m->ell_width > kMaxSlots || !m->ell_col)
        return WCFD_ERR_ARGUMENT;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    int nb = (m->n_cells + kBlock - 1) / kBlock;
    if (nb > kNormBlocks) nb = kNormBlocks;
    norms_partial_kernel<<<nb, kBlock, 0, st>>>(*m, A, x, div, cell_gradients, rua, p, scratch);
    norms_final_kernel<<<1, 32, 0, st>>>(nb, scratch, out);
    return cudaGetLastError() == cudaSuccess ? WCFD_OK : WCFD_ERR_CUDA;
}
