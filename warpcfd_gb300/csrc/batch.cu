// Host side of the batched form: one SIMPLE outer iteration (or PISO step) for every case
// of a device case table, as a fixed sequence of batched launches (capturable in a CUDA
// graph: the sequence depends only on the dims, never on the data).
#include <cstdio>
#include <mutex>

#include "common.cuh"
#include "kernels.cuh"

using namespace wcfd;

namespace {

thread_local char g_batch_error[256] = "";

inline cudaStream_t S(void* s) { return reinterpret_cast<cudaStream_t>(s); }

int batch_budget_rows(int W) {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return cluster_cg_max_rows(W, optin);
}

int pick_cluster(const wcfd_batch_dims& d) {
    const int rmax = batch_budget_rows(d.ell_width);
    for (int c = 1; c <= 16; c *= 2) {
        const long long r = (d.max_cells + c - 1) / c;
        if (r <= rmax && (r <= 2048 || c == 16)) return c;
    }
    return 0;
}

// the launch attributes a cluster kernel needs (dynamic shared memory, non-portable
// cluster size), set once per (kernel, device, size); 0 on success
int prepare_cluster(const void* fn, size_t smem) {
    static std::mutex mu;
    static size_t set_bytes[128] = {0};
    static const void* set_fn[128] = {nullptr};
    static int set_dev[128] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    {
        std::lock_guard<std::mutex> lk(mu);
        int slot = -1;
        for (int i = 0; i < 128; ++i)
            if ((set_fn[i] == fn && set_dev[i] == dev) || set_fn[i] == nullptr) {
                slot = i;
                break;
            }
        if (slot < 0) {
            std::snprintf(g_batch_error, sizeof(g_batch_error), "cluster kernel attribute cache full");
            return WCFD_ERR_CUDA;
        }
        if (set_fn[slot] == nullptr || set_bytes[slot] < smem) {
            if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
                cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
                std::snprintf(g_batch_error, sizeof(g_batch_error), "cluster kernel attributes: %s",
                              cudaGetErrorString(cudaGetLastError()));
                return WCFD_ERR_CUDA;
            }
            set_fn[slot] = fn;
            set_dev[slot] = dev;
            set_bytes[slot] = smem;
        }
    }
    return WCFD_OK;
}

int launch_cluster(const void* fn, int n_cases, int cs, size_t smem, cudaStream_t st, void** args) {
    const int rc = prepare_cluster(fn, smem);
    if (rc) return rc;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(n_cases * cs);
    cfg.blockDim = dim3(kClusterBlock);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cs;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelExC(&cfg, fn, args);
    if (e != cudaSuccess) {
        cudaGetLastError();
        std::snprintf(g_batch_error, sizeof(g_batch_error), "batched cluster launch: %s", cudaGetErrorString(e));
        return WCFD_ERR_CUDA;
    }
    return WCFD_OK;
}

// One refinement sweep's residual for every case: r = b - A x64 with fp64 accumulation,
// rounded once into p_work[0, C); the correction p_work[C, 2C) starts from zero.
__global__ void __launch_bounds__(kMaxFieldBlock) refine_residual_batched(const wcfd_case* __restrict__ cases) {
    const wcfd_case& c = cases[blockIdx.y];
    const int C = c.mesh.n_cells;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= C) return;
    const int W = c.mesh.ell_width;
    double acc = (double)c.pres.diag[i] * c.p_x64[i];
    for (int j = 0; j < W; ++j)
        acc += (double)c.pres.off[(size_t)j * C + i] * c.p_x64[c.mesh.ell_col[(size_t)j * C + i]];
    c.p_work[i] = (float)((double)c.pres.rhs[i] - acc);
    c.p_work[C + i] = 0.0f;
}

// x64 += the sweep's correction; the field solution p_x is x64 rounded once
__global__ void __launch_bounds__(kMaxFieldBlock) refine_update_batched(const wcfd_case* __restrict__ cases) {
    const wcfd_case& c = cases[blockIdx.y];
    const int C = c.mesh.n_cells;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= C) return;
    const double v = c.p_x64[i] + (double)c.p_work[C + i];
    c.p_x64[i] = v;
    c.p_x[i] = (float)v;
}

// the pressure CG of the batch: textbook (cg_variant 0) or single-reduction (1)
const void* batch_cg_kernel(const wcfd_batch_dims& d, int R) {
    return d.cg_variant == 1 ? cg1m_cluster_batched_for(d.ell_width, R) : cg_cluster_batched_for(d.ell_width, R);
}
size_t batch_cg_smem(const wcfd_batch_dims& d, int R) {
    return d.cg_variant == 1 ? cluster_cg1m_smem_bytes(R, d.ell_width) : cluster_cg_smem_bytes(R, d.ell_width);
}

#define BCHECK(what)                                                                               \
    do {                                                                                           \
        const cudaError_t e_ = cudaGetLastError();                                                 \
        if (e_ != cudaSuccess) {                                                                   \
            std::snprintf(g_batch_error, sizeof(g_batch_error), "%s: %s", what, cudaGetErrorString(e_)); \
            return WCFD_ERR_CUDA;                                                                  \
        }                                                                                          \
    } while (0)

}  // namespace

extern "C" const char* wcfd_batch_last_error(void) { return g_batch_error; }

extern "C" int wcfd_batch_prepare(const wcfd_batch_dims* dims) {
    if (!dims || dims->max_cells <= 0 || dims->ell_width < 0 || dims->ell_width > kMaxSlots) return WCFD_ERR_ARGUMENT;
    const int cs = dims->cluster_size > 0 ? dims->cluster_size : pick_cluster(*dims);
    if (cs < 1 || cs > 16) return WCFD_ERR_TOO_LARGE;
    if (dims->cg_variant != 0 && dims->cg_variant != 1) return WCFD_ERR_ARGUMENT;
    const int R = (dims->max_cells + cs - 1) / cs;
    const void* cg_fn = batch_cg_kernel(*dims, R);
    const void* bi_fn = bicgstab_cluster_batched_for(dims->ell_width);
    if (!cg_fn || !bi_fn) return WCFD_ERR_ARGUMENT;
    int rc = prepare_cluster(bi_fn, 0);
    if (!rc) rc = prepare_cluster(cg_fn, batch_cg_smem(*dims, R));
    return rc;
}

extern "C" int wcfd_batch_max_rows(int32_t ell_width) {
    if (ell_width < 0 || ell_width > kMaxSlots) return 0;
    return batch_budget_rows(ell_width);
}

extern "C" int wcfd_batch_cluster_size(const wcfd_batch_dims* dims) {
    if (!dims || dims->max_cells <= 0 || dims->ell_width < 0 || dims->ell_width > kMaxSlots) return 0;
    return pick_cluster(*dims);
}

extern "C" int wcfd_batch_simple_iteration(const wcfd_case* cases, int32_t n_cases, const wcfd_batch_dims* dims,
                                           void* stream) {
    if (!cases || !dims || n_cases <= 0) {
        std::snprintf(g_batch_error, sizeof(g_batch_error), "null case table, dims or empty batch");
        return WCFD_ERR_ARGUMENT;
    }
    const wcfd_batch_dims d = *dims;
    if (d.max_cells <= 0 || d.max_faces <= 0 || d.faces_per_cell < 1 || d.faces_per_cell > kMaxSlots ||
        d.ell_width < 0 || d.ell_width > d.faces_per_cell || d.n_inner < 0 || d.n_ortho < 0 || n_cases > 65535 ||
        d.p_refine < 0 || d.p_refine > 64 || (d.cg_variant != 0 && d.cg_variant != 1)) {
        std::snprintf(g_batch_error, sizeof(g_batch_error), "bad batch dims");
        return WCFD_ERR_ARGUMENT;
    }
    const int fb = d.field_block > 0 ? d.field_block : kBlock;
    if (fb < 64 || fb > kMaxFieldBlock || fb % 32 != 0) {
        std::snprintf(g_batch_error, sizeof(g_batch_error), "field_block must be 64..%d in steps of 32", kMaxFieldBlock);
        return WCFD_ERR_ARGUMENT;
    }
    const int cs = d.cluster_size > 0 ? d.cluster_size : pick_cluster(d);
    if (cs < 1 || cs > 16) {
        std::snprintf(g_batch_error, sizeof(g_batch_error), "no cluster size fits max_cells %d", d.max_cells);
        return WCFD_ERR_TOO_LARGE;
    }
    const int R = (d.max_cells + cs - 1) / cs;
    if (R > batch_budget_rows(d.ell_width)) {
        std::snprintf(g_batch_error, sizeof(g_batch_error), "max_cells %d too large for cluster size %d", d.max_cells, cs);
        return WCFD_ERR_TOO_LARGE;
    }
    const void* cg_fn = batch_cg_kernel(d, R);
    const void* bi_fn = bicgstab_cluster_batched_for(d.ell_width);
    if (!cg_fn || !bi_fn) return WCFD_ERR_ARGUMENT;
    cudaStream_t st = S(stream);
    NvtxRange step_range("wcfd batched iteration");
    const dim3 gf((d.max_faces + fb - 1) / fb, n_cases), gc((d.max_cells + fb - 1) / fb, n_cases);
    // incompressible.py:96-99
    face_pass_batched<<<gf, fb, 0, st>>>(cases, WCFD_ALL, 1u | 2u);
    BCHECK("face_pass_batched");
    gradient_batched<<<gc, fb, 0, st>>>(cases, WCFD_ALL, 0);
    BCHECK("gradient_batched");
    // :102-116
    launch_assemble_batched(false, d.explicit_terms != 0, gc, fb, st, cases);
    BCHECK("momentum_assemble_batched");
    int csv = cs;
    void* bargs[] = {(void*)&cases, &csv};
    int rc = launch_cluster(bi_fn, n_cases, cs, 0, st, bargs);
    if (rc) return rc;
    // :118-123
    hbya_batched<<<gc, fb, 0, st>>>(cases);
    BCHECK("hbya_batched");
    rua_faces_batched<<<gf, fb, 0, st>>>(cases);
    BCHECK("rua_faces_batched");
    const size_t smem = batch_cg_smem(d, R);
    for (int inner = 0; inner < d.n_inner; ++inner) {
        for (int ortho = 0; ortho < d.n_ortho; ++ortho) {
            face_pass_batched<<<gf, fb, 0, st>>>(cases, WCFD_ALL, 2u);
            BCHECK("face_pass_batched");
            gradient_batched<<<gc, fb, 0, st>>>(cases, WCFD_ALL, 1);
            BCHECK("gradient_batched");
            launch_assemble_batched(true, (d.explicit_terms & 4) != 0, gc, fb, st, cases);
            BCHECK("pressure_assemble_batched");
            if (d.p_refine > 0) {
                int one = 1;
                for (int sw = 0; sw < d.p_refine; ++sw) {
                    refine_residual_batched<<<gc, fb, 0, st>>>(cases);
                    BCHECK("refine_residual_batched");
                    void* cargs[] = {(void*)&cases, &csv, &one};
                    rc = launch_cluster(cg_fn, n_cases, cs, smem, st, cargs);
                    if (rc) return rc;
                    refine_update_batched<<<gc, fb, 0, st>>>(cases);
                    BCHECK("refine_update_batched");
                }
            } else {
                int zero = 0;
                void* cargs[] = {(void*)&cases, &csv, &zero};
                rc = launch_cluster(cg_fn, n_cases, cs, smem, st, cargs);
                if (rc) return rc;
            }
            p_update_batched<<<gc, fb, 0, st>>>(cases);
            BCHECK("p_update_batched");
            face_pass_partial_batched<<<gf, fb, 0, st>>>(cases, WCFD_P, 0u);
            BCHECK("face_pass_partial_batched");
            gradient_batched<<<gc, fb, 0, st>>>(cases, WCFD_P, 2);
            BCHECK("gradient_batched");
        }
    }
    return WCFD_OK;
}
