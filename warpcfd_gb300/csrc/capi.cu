// extern "C" entry points of libwcfd.so (declared in include/wcfd.h).
#include <cstdio>
#include <cstring>
#include <mutex>

#include "common.cuh"
#include "kernels.cuh"

using namespace wcfd;

// rows per block the grid-cooperative Krylov kernels are sized for (capped at the blocks
// that can be co-resident)
#ifndef WCFD_GRID_ROWS_PER_BLOCK
#define WCFD_GRID_ROWS_PER_BLOCK 1024
#endif

namespace {

thread_local char g_last_error[512] = "";

int set_error(int code, const char* what) {
    std::snprintf(g_last_error, sizeof(g_last_error), "%s", what);
    return code;
}

int check_launch(const char* what) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s", what, cudaGetErrorString(e));
        return WCFD_ERR_CUDA;
    }
    return WCFD_OK;
}

#define RET_IF(cond, code, msg) \
    do {                        \
        if (cond) return set_error(code, msg); \
    } while (0)
#define LAUNCH_CHECK(what)                 \
    do {                                   \
        const int rc_ = check_launch(what); \
        if (rc_ != WCFD_OK) return rc_;     \
    } while (0)

int check_mesh(const wcfd_mesh* m) {
    if (!m) return set_error(WCFD_ERR_ARGUMENT, "mesh is null");
    if (m->n_cells <= 0 || m->n_faces <= 0) return set_error(WCFD_ERR_ARGUMENT, "empty mesh");
    if (m->faces_per_cell < 1 || m->faces_per_cell > kMaxSlots)
        return set_error(WCFD_ERR_ARGUMENT, "faces_per_cell must be in 1..6");
    if (m->ell_width < 0 || m->ell_width > m->faces_per_cell)
        return set_error(WCFD_ERR_ARGUMENT, "ell_width must be in 0..faces_per_cell");
    if (!m->face_owner || !m->face_nbr || !m->face_brow || !m->face_interp || !m->face_normal ||
        !m->face_gdiff || !m->face_rpf || !m->cell_slot || !m->cell_volume || !m->ell_col)
        return set_error(WCFD_ERR_ARGUMENT, "mesh has a null array");
    return WCFD_OK;
}

inline cudaStream_t S(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// co-resident blocks of a cooperative kernel on the current device (cached per kernel
// and device)
int coop_capacity(const void* fn, int /*unused*/) {
    static std::mutex mu;
    struct Entry { const void* fn; int dev; int cap; };
    static Entry cache[64];
    static int n = 0;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(mu);
    for (int i = 0; i < n; ++i)
        if (cache[i].fn == fn && cache[i].dev == dev) return cache[i].cap;
    int per_sm = 0, sms = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kSolverBlock, 0);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int cap = per_sm * sms;
    if (cap > WCFD_MAX_BLOCKS) cap = WCFD_MAX_BLOCKS;
    if (cap > kSolverBlock) cap = kSolverBlock;  // grid_sync: one waiting thread per block
    if (n < 64) cache[n++] = Entry{fn, dev, cap};
    return cap;
}

// Grid of a persistent kBlock-thread kernel over n items: every block resident at once
// (blocks per SM from the occupancy query, cached per kernel and device), fewer when
// there are fewer items than resident threads.
int resident_grid(const void* fn, long long n) {
    static std::mutex mu;
    struct Entry { const void* fn; int dev; int cap; };
    static Entry cache[16];
    static int nc = 0;
    int dev = 0;
    cudaGetDevice(&dev);
    int cap = 0;
    {
        std::lock_guard<std::mutex> lk(mu);
        for (int i = 0; i < nc; ++i)
            if (cache[i].fn == fn && cache[i].dev == dev) cap = cache[i].cap;
        if (cap == 0) {
            int per_sm = 0, sms = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kBlock, 0);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            cap = per_sm * sms;
            if (cap < 1) cap = 1;
            if (nc < 16) cache[nc++] = Entry{fn, dev, cap};
        }
    }
    const int want = grid_for(n);
    return want < cap ? (want < 1 ? 1 : want) : cap;
}

int launch_krylov(const void* fn, int slot, const wcfd_mesh* m, wcfd_system A, float* x, wcfd_krylov_ws ws,
                  double atol, int maxiter, wcfd_solve_stats* stats, cudaStream_t st, const char* name,
                  double rtol = 0.0) {
    int rc = check_mesh(m);
    if (rc) return rc;
    RET_IF(!fn, WCFD_ERR_ARGUMENT, "no solver kernel for this off-diagonal width");
    RET_IF(!A.diag || !A.off || !A.rhs || !x || !ws.vec || !ws.partials || !ws.barrier || !stats,
           WCFD_ERR_ARGUMENT, "null solver argument");
    // the grid barrier stores each block's partial sums as one float4
    RET_IF(reinterpret_cast<uintptr_t>(ws.partials) % 16 != 0, WCFD_ERR_ARGUMENT,
           "Krylov workspace: partials must be 16-byte aligned");
    RET_IF(maxiter < 0 || !(atol >= 0.0), WCFD_ERR_ARGUMENT, "bad atol or maxiter");
    const int cap = coop_capacity(fn, slot);
    LAUNCH_CHECK("occupancy query");
    RET_IF(cap <= 0, WCFD_ERR_CUDA, "solver kernel cannot be resident");
    long long want = (m->n_cells + WCFD_GRID_ROWS_PER_BLOCK - 1) / WCFD_GRID_ROWS_PER_BLOCK;
    int grid = (int)(want < cap ? want : cap);
    if (grid < 1) grid = 1;
    if (cudaMemsetAsync(ws.barrier, 0, WCFD_BARRIER_WORDS * sizeof(uint32_t), st) != cudaSuccess)
        return set_error(WCFD_ERR_CUDA, "barrier reset failed");
    KrylovArgs a = {};
    a.m = *m;
    a.A = A;
    a.x = x;
    a.ws = ws.vec;
    a.g.partials = ws.partials;
    a.g.flags = ws.barrier;
    a.g.err = reinterpret_cast<int*>(ws.barrier + WCFD_MAX_BLOCKS);
    a.atol2 = atol * atol;
    a.rtol2 = rtol * rtol;
    a.maxiter = maxiter;
    a.stats = stats;
    void* args[] = {&a};
    const cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(kSolverBlock), args, 0, st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s", name, cudaGetErrorString(e));
        return WCFD_ERR_CUDA;
    }
    return WCFD_OK;
}

int g_krylov_path = 0;  // 0 automatic, 1 grid-cooperative only, 2 cluster-resident when it fits, 3 as 2 with the single-reduction CG

// the cluster CG takes the smallest cluster whose CTAs hold at most this many rows each
// (larger systems take 16 CTAs).  Its iteration is bound by the cluster reductions, so
// more CTAs with fewer rows per thread are faster down to ~512 rows per CTA (measured on a
// 4,096-row system: 2,048 rows per CTA 120 us per solve, 1,024 108, 512 106, 256 113)
#ifndef WCFD_CLUSTER_ROW_CAP
#define WCFD_CLUSTER_ROW_CAP 512
#endif

// Cluster-resident CG when the system fits in the shared memory of one cluster of up to
// 16 CTAs; returns -1 (caller falls back to the grid-cooperative kernel) otherwise.
int try_cluster_cg(const wcfd_mesh* m, wcfd_system A, float* x, double atol, int maxiter,
                   wcfd_solve_stats* stats, cudaStream_t st, double rtol = 0.0) {
    if (g_krylov_path == 1) return -1;
    const int C = m->n_cells, W = m->ell_width;
    int dev = 0;
    cudaGetDevice(&dev);
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const int rmax = cluster_cg_max_rows(W, optin);
    int cs = 0, R = 0;
    for (int c = 1; c <= 16; c *= 2) {
        const long long r = (C + c - 1) / c;
        if (r <= rmax && (r <= WCFD_CLUSTER_ROW_CAP || c == 16)) {
            cs = c;
            R = (int)r;
            break;
        }
    }
    if (cs == 0) return -1;
    // the textbook kernel; the single-reduction arrangement when asked for (path 3) and its
    // registers (<= 2 rows per thread) and shared memory allow
    size_t smem = cluster_cg_smem_bytes(R, W);
    const void* fn = cg_cluster_kernel_for(W, R);
    const size_t smem1 = cluster_cg1_smem_bytes(R, W);
    if (g_krylov_path == 3 && R <= 2 * kClusterBlock && smem1 + 2048 <= (size_t)optin) {
        fn = cg1_cluster_kernel_for(W, R);
        smem = smem1;
    }
    if (!fn) return -1;
    static std::mutex mu;
    struct SetA { const void* fn; int dev; size_t bytes; };
    static SetA set_attr[128];
    static int n_set = 0;
    {
        std::lock_guard<std::mutex> lk(mu);
        int slot = -1;
        for (int i = 0; i < n_set; ++i)
            if (set_attr[i].fn == fn && set_attr[i].dev == dev) slot = i;
        if (slot < 0 || set_attr[slot].bytes < smem) {
            if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
                cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
                cudaGetLastError();
                return -1;
            }
            if (slot < 0 && n_set < 128) slot = n_set++;
            if (slot >= 0) set_attr[slot] = SetA{fn, dev, smem};
        }
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cs);
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
    // whether this (device, size, width) cluster launch is schedulable, asked once
    static std::mutex qmu;
    struct Q { int dev, C; const void* fn; int ok; };
    static Q qcache[64];
    static int nq = 0;
    int ok = -1;
    {
        std::lock_guard<std::mutex> lk(qmu);
        for (int i = 0; i < nq; ++i)
            if (qcache[i].dev == dev && qcache[i].C == C && qcache[i].fn == fn) ok = qcache[i].ok;
        if (ok < 0) {
            int nclusters = 0;
            ok = (cudaOccupancyMaxActiveClusters(&nclusters, fn, &cfg) == cudaSuccess && nclusters >= 1) ? 1 : 0;
            cudaGetLastError();
            if (nq < 64) qcache[nq++] = Q{dev, C, fn, ok};
        }
    }
    if (!ok) return -1;
    KrylovArgs a = {};
    a.m = *m;
    a.A = A;
    a.x = x;
    a.atol2 = atol * atol;
    a.rtol2 = rtol * rtol;
    a.maxiter = maxiter;
    a.stats = stats;
    void* args[] = {&a, &R};
    const cudaError_t e = cudaLaunchKernelExC(&cfg, fn, args);
    if (e != cudaSuccess) {
        cudaGetLastError();
        std::snprintf(g_last_error, sizeof(g_last_error), "cg_cluster_kernel: %s", cudaGetErrorString(e));
        return WCFD_ERR_CUDA;
    }
    return WCFD_OK;
}

}  // namespace

extern "C" {

int wcfd_version(void) { return 100; }

int wcfd_set_krylov_path(int32_t path) {
    if (path < 0 || path > 3)
        return set_error(WCFD_ERR_ARGUMENT,
                         "path must be 0 (auto), 1 (grid), 2 (cluster), 3 (cluster, single-reduction CG)");
    g_krylov_path = path;
    return WCFD_OK;
}

const char* wcfd_last_error(void) { return g_last_error; }

int wcfd_grid_barrier_check(int32_t skip_block, int32_t phases, int32_t* result, void* stream) {
    RET_IF(!result || phases < 1 || phases > 100000, WCFD_ERR_ARGUMENT, "bad phases or null result");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const void* fn = barrier_check_kernel_ptr();
    const int cap = coop_capacity(fn, 0);
    LAUNCH_CHECK("occupancy query");
    RET_IF(cap <= 0, WCFD_ERR_CUDA, "barrier check kernel cannot be resident");
    RET_IF(skip_block >= cap, WCFD_ERR_ARGUMENT, "skip_block beyond the grid");
    unsigned* words = nullptr;
    double* partials = nullptr;
    int* bad = nullptr;
    int rc = WCFD_OK;
    if (cudaMalloc(&words, WCFD_BARRIER_WORDS * sizeof(unsigned)) != cudaSuccess ||
        cudaMalloc(&partials, 8 * WCFD_MAX_BLOCKS * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&bad, sizeof(int)) != cudaSuccess) {
        rc = set_error(WCFD_ERR_CUDA, "barrier check: allocation failed");
    }
    if (rc == WCFD_OK && (cudaMemsetAsync(words, 0, WCFD_BARRIER_WORDS * sizeof(unsigned), st) != cudaSuccess ||
                          cudaMemsetAsync(bad, 0, sizeof(int), st) != cudaSuccess))
        rc = set_error(WCFD_ERR_CUDA, "barrier check: memset failed");
    if (rc == WCFD_OK) {
        GridCtl g;
        g.partials = partials;
        g.flags = words;
        g.err = reinterpret_cast<int*>(words + WCFD_MAX_BLOCKS);
        int skip = skip_block, ph = phases;
        void* args[] = {&g, &skip, &ph, &bad};
        int host[2] = {0, 0};
        if (cudaLaunchCooperativeKernel(fn, dim3(cap), dim3(kSolverBlock), args, 0, st) != cudaSuccess ||
            cudaMemcpyAsync(&host[0], g.err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaMemcpyAsync(&host[1], bad, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            rc = check_launch("barrier check");
            if (rc == WCFD_OK) rc = set_error(WCFD_ERR_CUDA, "barrier check failed");
        } else {
            result[0] = host[0];
            result[1] = host[1];
            result[2] = cap;
        }
    }
    cudaFree(words);
    cudaFree(partials);
    cudaFree(bad);
    return rc;
}

int64_t wcfd_krylov_workspace_floats(int32_t n_cells, int32_t ncomp) {
    if (n_cells <= 0 || (ncomp != 1 && ncomp != 3)) return -1;
    return ncomp == 1 ? 6LL * n_cells : 27LL * n_cells;
}

int wcfd_face_pass_flags(const wcfd_mesh* m, wcfd_bc bc, wcfd_state s, uint32_t mask, uint32_t flags,
                         void* stream) {
    int rc = check_mesh(m);
    if (rc) return rc;
    RET_IF(mask > WCFD_ALL || flags > 15u, WCFD_ERR_ARGUMENT, "bad mask or flags");
    RET_IF(!bc.type || !bc.value || !s.cell_values || !s.cell_gradients || !s.face_values || !s.face_gradients ||
               !s.mass_fluxes,
           WCFD_ERR_ARGUMENT, "null field");
    if (mask == WCFD_ALL)
        face_pass_kernel<<<resident_grid((const void*)face_pass_kernel, m->n_faces), kBlock, 0, S(stream)>>>(
            *m, bc, s, mask, flags & 15u, nullptr);
    else
        face_pass_partial_kernel<<<resident_grid((const void*)face_pass_partial_kernel, m->n_faces), kBlock, 0, S(stream)>>>(
            *m, bc, s, mask, flags & 15u, nullptr);
    LAUNCH_CHECK("face_pass_kernel");
    return WCFD_OK;
}

int wcfd_set_boundary_conditions(const wcfd_mesh* m, wcfd_bc bc, wcfd_state s, void* stream) {
    return wcfd_face_pass_flags(m, bc, s, 0u, 1u, stream);
}

int wcfd_face_interpolation(const wcfd_mesh* m, wcfd_bc bc, wcfd_state s, uint32_t mask, int32_t skew,
                            int32_t upwind, void* stream) {
    return wcfd_face_pass_flags(m, bc, s, mask, (skew ? 4u : 0u) | (upwind ? 8u : 0u), stream);
}

int wcfd_calculate_mass_flux(const wcfd_mesh* m, wcfd_state s, void* stream) {
    int rc = check_mesh(m);
    if (rc) return rc;
    RET_IF(!s.face_values || !s.mass_fluxes, WCFD_ERR_ARGUMENT, "null field");
    mass_flux_kernel<<<grid_for(m->n_faces), kBlock, 0, S(stream)>>>(*m, s);
    LAUNCH_CHECK("mass_flux_kernel");
    return WCFD_OK;
}

int wcfd_calculate_gradients(const wcfd_mesh* m, wcfd_state s, uint32_t mask, void* stream) {
    int rc = check_mesh(m);
    if (rc) return rc;
    RET_IF(mask > WCFD_ALL, WCFD_ERR_ARGUMENT, "bad mask");
    RET_IF(!s.cell_gradients || !s.face_values, WCFD_ERR_ARGUMENT, "null field");
    gradient_kernel<<<grid_for(m->n_cells), kBlock, 0, S(stream)>>>(*m, s, mask, nullptr, CorrectArgs{nullptr, nullptr});
    LAUNCH_CHECK("gradient_kernel");
    return WCFD_OK;
}

int wcfd_div_flux(const wcfd_mesh* m, const float* mass_fluxes, float* div, void* stream) {
    int rc = check_mesh(m);
    if (rc) return rc;
    RET_IF(!mass_fluxes || !div, WCFD_ERR_ARGUMENT, "null array");
    div_kernel<<<grid_for(m->n_cells), kBlock, 0, S(stream)>>>(*m, mass_fluxes, div);
    LAUNCH_CHECK("div_kernel");
    return WCFD_OK;
}

int wcfd_cell_to_face(const wcfd_mesh* m, const float* cell, float* face, void* stream) {
    int rc = check_mesh(m);
    if (rc) return rc;
    RET_IF(!cell || !face, WCFD_ERR_ARGUMENT, "null array");
    cell_to_face_kernel<<<resident_grid((const void*)cell_to_face_kernel, m->n_faces), kBlock, 0, S(stream)>>>(*m, cell, face);
    LAUNCH_CHECK("cell_to_face_kernel");
    return WCFD_OK;
}

int wcfd_rua(const wcfd_mesh* m, const float* diag3, float rho, float* rua, void* stream) {
    int rc = check_mesh(m);
    if (rc) return rc;
    RET_IF(!diag3 || !rua || rho == 0.0f, WCFD_ERR_ARGUMENT, "null array or zero density");
    rua_kernel<<<grid_for(m->n_cells), kBlock, 0, S(stream)>>>(m->n_cells, m->cell_volume, diag3, rho, rua);
    LAUNCH_CHECK("rua_kernel");
    return WCFD_OK;
}

int wcfd_hbya_add(int32_t n_cells, const float* pgrad3, const float* rua, float* hbya, void* stream) {
    RET_IF(n_cells <= 0 || !pgrad3 || !rua || !hbya, WCFD_ERR_ARGUMENT, "bad arguments");
    hbya_add_kernel<<<grid_for(n_cells), kBlock, 0, S(stream)>>>(n_cells, pgrad3, rua, hbya);
    LAUNCH_CHECK("hbya_add_kernel");
    return WCFD_OK;
}

int wcfd_assemble_momentum(const wcfd_case* c, void* stream) {
    RET_IF(!c, WCFD_ERR_ARGUMENT, "case is null");
    int rc = check_mesh(&c->mesh);
    if (rc) return rc;
    RET_IF(!c->mom.diag || !c->mom.off || !c->mom.rhs || !c->rua, WCFD_ERR_ARGUMENT, "null momentum array");
    RET_IF(c->prm.rho == 0.0f || (!c->prm.steady && c->prm.dt <= 0.0f), WCFD_ERR_ARGUMENT, "bad rho or dt");
    launch_momentum_assemble(c->prm.explicit_terms != 0, grid_for(c->mesh.n_cells), S(stream), c->mesh, c->bc,
                             c->state, c->mom, c->rua, c->prm);
    LAUNCH_CHECK("momentum_assemble_kernel");
    return WCFD_OK;
}

int wcfd_assemble_pressure(const wcfd_case* c, void* stream) {
    RET_IF(!c, WCFD_ERR_ARGUMENT, "case is null");
    int rc = check_mesh(&c->mesh);
    if (rc) return rc;
    RET_IF(!c->pres.diag || !c->pres.off || !c->pres.rhs || !c->rua_faces || !c->div, WCFD_ERR_ARGUMENT,
           "null pressure array");
    RET_IF(c->prm.ref_cell >= c->mesh.n_cells, WCFD_ERR_ARGUMENT, "reference cell out of range");
    launch_pressure_assemble((c->prm.explicit_terms & 4) != 0, grid_for(c->mesh.n_cells), S(stream), c->mesh, c->bc,
                             c->state, c->pres, c->rua_faces, c->div, c->prm);
    LAUNCH_CHECK("pressure_assemble_kernel");
    return WCFD_OK;
}

int wcfd_relax(const wcfd_mesh* m, wcfd_system A, const float* cell_values, int32_t field0, float alpha,
               void* stream) {
    int rc = check_mesh(m);
    if (rc) return rc;
    RET_IF(!A.diag || !A.rhs || !cell_values || (A.ncomp != 1 && A.ncomp != 3), WCFD_ERR_ARGUMENT, "bad system");
    RET_IF(field0 < 0 || field0 + A.ncomp > 4, WCFD_ERR_ARGUMENT, "fields out of range");
    RET_IF(!(alpha > 0.0f && alpha <= 1.0f), WCFD_ERR_ARGUMENT, "relaxation factor must be in (0, 1]");
    relax_kernel<<<grid_for(m->n_cells), kBlock, 0, S(stream)>>>(m->n_cells, A, cell_values, field0, alpha);
    LAUNCH_CHECK("relax_kernel");
    return WCFD_OK;
}

int wcfd_replace_row(const wcfd_mesh* m, wcfd_system A, int32_t row, float value, void* stream) {
    int rc = check_mesh(m);
    if (rc) return rc;
    RET_IF(!A.diag || !A.off || !A.rhs || A.ncomp != 1, WCFD_ERR_ARGUMENT, "replace_row takes a scalar system");
    RET_IF(row < 0 || row >= m->n_cells, WCFD_ERR_ARGUMENT, "row out of range");
    replace_row_kernel<<<1, 32, 0, S(stream)>>>(m->n_cells, m->ell_width, A, row, value);
    LAUNCH_CHECK("replace_row_kernel");
    return WCFD_OK;
}

static int check_term_fields(const wcfd_term_fields& f) {
    RET_IF(f.n < 1 || f.n > 3, WCFD_ERR_ARGUMENT, "a term acts on 1..3 fields");
    for (int q = 0; q < f.n; ++q) RET_IF(f.index[q] < 0 || f.index[q] > 3, WCFD_ERR_ARGUMENT, "field index out of 0..3");
    return WCFD_OK;
}

static int grid_slots(const wcfd_mesh* m) { return (m->n_cells * m->faces_per_cell + kBlock - 1) / kBlock; }

int wcfd_convection_weights(const wcfd_mesh* m, wcfd_state s, wcfd_term_fields f, int32_t scheme, float* weights,
                            void* stream) {
    int rc = check_mesh(m);
    if (rc) return rc;
    rc = check_term_fields(f);
    if (rc) return rc;
    RET_IF(scheme < 0 || scheme > 2, WCFD_ERR_ARGUMENT, "convection scheme must be 0 upwind, 1 central, 2 upwindLinear");
    RET_IF(!weights || !s.mass_fluxes || !s.face_values || !s.cell_gradients || !m->face_dvec, WCFD_ERR_ARGUMENT,
           "null array");
    convection_weights_kernel<<<grid_slots(m), kBlock, 0, S(stream)>>>(*m, s, f, scheme, weights);
    LAUNCH_CHECK("convection_weights_kernel");
    return WCFD_OK;
}

int wcfd_diffusion_weights(const wcfd_mesh* m, wcfd_bc bc, wcfd_state s, wcfd_term_fields f, float nu,
                           const float* nu_faces, int32_t corrected, int32_t bc_mode, float bc_value, float* weights,
                           void* stream) {
    int rc = check_mesh(m);
    if (rc) return rc;
    rc = check_term_fields(f);
    if (rc) return rc;
    RET_IF(bc_mode != 0 && bc_mode != 1, WCFD_ERR_ARGUMENT, "bc_mode must be 0 (boundary table) or 1 (uniform gradient)");
    RET_IF(!weights || !s.face_values || !s.face_gradients || !s.cell_gradients || !m->face_dvec ||
           (bc_mode == 0 && !bc.type), WCFD_ERR_ARGUMENT, "null array");
    diffusion_weights_kernel<<<grid_slots(m), kBlock, 0, S(stream)>>>(*m, bc, s, f, nu, nu_faces, corrected, bc_mode,
                                                                       bc_value, weights);
    LAUNCH_CHECK("diffusion_weights_kernel");
    return WCFD_OK;
}

int wcfd_ddt_weights(const wcfd_mesh* m, wcfd_state s, wcfd_term_fields f, float dt, float* weights, void* stream) {
    int rc = check_mesh(m);
    if (rc) return rc;
    rc = check_term_fields(f);
    if (rc) return rc;
    RET_IF(!(dt > 0.0f), WCFD_ERR_ARGUMENT, "dt must be positive");
    RET_IF(!weights || !s.cell_values, WCFD_ERR_ARGUMENT, "null array");
    ddt_weights_kernel<<<grid_for(m->n_cells * f.n), kBlock, 0, S(stream)>>>(*m, s, f, dt, weights);
    LAUNCH_CHECK("ddt_weights_kernel");
    return WCFD_OK;
}

int wcfd_grad_weights(const wcfd_mesh* m, wcfd_state s, int32_t field, float* weights, void* stream) {
    int rc = check_mesh(m);
    if (rc) return rc;
    RET_IF(field < 0 || field > 3, WCFD_ERR_ARGUMENT, "field index out of 0..3");
    RET_IF(!weights || !s.cell_gradients, WCFD_ERR_ARGUMENT, "null array");
    grad_weights_kernel<<<grid_for(3 * m->n_cells), kBlock, 0, S(stream)>>>(*m, s, field, weights);
    LAUNCH_CHECK("grad_weights_kernel");
    return WCFD_OK;
}

int wcfd_assemble_terms(const wcfd_mesh* m, wcfd_system A, const wcfd_term* terms, int32_t n_terms, void* stream) {
    int rc = check_mesh(m);
    if (rc) return rc;
    RET_IF(!A.diag || !A.off || !A.rhs || (A.ncomp != 1 && A.ncomp != 3), WCFD_ERR_ARGUMENT, "bad system");
    RET_IF(n_terms < 0 || n_terms > WCFD_MAX_TERMS || (n_terms > 0 && !terms), WCFD_ERR_ARGUMENT,
           "0..WCFD_MAX_TERMS terms");
    TermList tl = {};
    tl.count = n_terms;
    for (int t = 0; t < n_terms; ++t) {
        RET_IF(!terms[t].weights, WCFD_ERR_ARGUMENT, "a term without weights (call the term first)");
        tl.weights[t] = terms[t].weights;
        tl.scale[t] = terms[t].scale;
        tl.cell_based[t] = terms[t].cell_based ? 1 : 0;
    }
    assemble_terms_kernel<<<grid_for(m->n_cells), kBlock, 0, S(stream)>>>(*m, A, tl);
    LAUNCH_CHECK("assemble_terms_kernel");
    return WCFD_OK;
}

int wcfd_add_rhs(float* rhs, const float* arr, float scale, int64_t n, void* stream) {
    RET_IF(n < 0 || (n > 0 && (!rhs || !arr)), WCFD_ERR_ARGUMENT, "bad arrays");
    if (n == 0) return WCFD_OK;
    add_rhs_kernel<<<(unsigned)((n + kBlock - 1) / kBlock), kBlock, 0, S(stream)>>>(n, rhs, arr, scale);
    LAUNCH_CHECK("add_rhs_kernel");
    return WCFD_OK;
}

int wcfd_spmv(const wcfd_mesh* m, wcfd_system A, const float* x, float* y, void* stream) {
    int rc = check_mesh(m);
    if (rc) return rc;
    RET_IF(!A.diag || !A.off || !x || !y, WCFD_ERR_ARGUMENT, "null array");
    RET_IF(A.ncomp != 1 && A.ncomp != 3, WCFD_ERR_ARGUMENT, "ncomp must be 1 or 3");
    launch_spmv(*m, A, x, y, S(stream));
    LAUNCH_CHECK("spmv_kernel");
    return WCFD_OK;
}

static int cg_solve(const wcfd_mesh* m, wcfd_system A, float* x, wcfd_krylov_ws ws, double atol, double rtol,
                    int32_t maxiter, wcfd_solve_stats* stats, void* stream) {
    RET_IF(A.ncomp != 1, WCFD_ERR_ARGUMENT, "cg solves scalar systems (ncomp 1)");
    int rc = check_mesh(m);
    if (rc) return rc;
    RET_IF(!A.diag || !A.off || !A.rhs || !x || !stats, WCFD_ERR_ARGUMENT, "null solver argument");
    RET_IF(maxiter < 0 || !(atol >= 0.0) || !(rtol >= 0.0), WCFD_ERR_ARGUMENT, "bad tolerance or maxiter");
    rc = try_cluster_cg(m, A, x, atol, maxiter, stats, S(stream), rtol);
    if (rc >= 0) return rc;
    return launch_krylov(cg_kernel_for(m->ell_width, m->ell_dcol != nullptr), 0, m, A, x, ws, atol, maxiter, stats, S(stream), "cg_kernel",
                         rtol);
}

int wcfd_cg(const wcfd_mesh* m, wcfd_system A, float* x, wcfd_krylov_ws ws, double atol, int32_t maxiter,
            wcfd_solve_stats* stats, void* stream) {
    return cg_solve(m, A, x, ws, atol, 0.0, maxiter, stats, stream);
}

int wcfd_cg_refine(const wcfd_mesh* m, wcfd_system A, double* x64, float* x32, float* work, wcfd_krylov_ws ws,
                   int32_t sweeps, double inner_rtol, int32_t maxiter, wcfd_solve_stats* stats, void* stream) {
    int rc = check_mesh(m);
    if (rc) return rc;
    RET_IF(!x64 || !x32 || !work || sweeps < 1 || !(inner_rtol > 0.0 && inner_rtol < 1.0), WCFD_ERR_ARGUMENT,
           "bad refinement arguments");
    const void* res_fn = residual64_kernel_for(m->ell_width);
    RET_IF(!res_fn, WCFD_ERR_ARGUMENT, "no residual kernel for this width");
    cudaStream_t st = S(stream);
    const int C = m->n_cells;
    float* r = work;
    float* d = work + C;
    wcfd_system Ar = A;
    Ar.rhs = r;
    const int gc = grid_for(C);
    for (int sw = 0; sw < sweeps; ++sw) {
        wcfd_mesh mm = *m;
        void* rargs[] = {&mm, &A, &x64, &r};
        if (cudaLaunchKernel(res_fn, dim3(gc), dim3(kBlock), rargs, 0, st) != cudaSuccess) {
            LAUNCH_CHECK("residual64_kernel");
        }
        if (cudaMemsetAsync(d, 0, sizeof(float) * (size_t)C, st) != cudaSuccess)
            return set_error(WCFD_ERR_CUDA, "refinement memset failed");
        rc = cg_solve(m, Ar, d, ws, 0.0, inner_rtol, maxiter, stats, stream);
        if (rc) return rc;
        refine_update_kernel<<<gc, kBlock, 0, st>>>(C, x64, d, x32);
        LAUNCH_CHECK("refine_update_kernel");
        refine_count_kernel<<<1, 1, 0, st>>>(stats, reinterpret_cast<int*>(work + 2 * (size_t)C), sw == 0,
                                             sw == sweeps - 1);
        LAUNCH_CHECK("refine_count_kernel");
    }
    return WCFD_OK;
}

static int bicgstab_solve(const wcfd_mesh* m, wcfd_system A, float* x, wcfd_krylov_ws ws, double atol, double rtol,
                          int32_t maxiter, wcfd_solve_stats* stats, void* stream) {
    RET_IF(A.ncomp != 3, WCFD_ERR_ARGUMENT, "bicgstab solves the 3-component momentum system (ncomp 3)");
    RET_IF(!(rtol >= 0.0), WCFD_ERR_ARGUMENT, "bad rtol");
    return launch_krylov(bicgstab_kernel_for(m->ell_width), 1, m, A, x, ws, atol, maxiter, stats, S(stream),
                         "bicgstab_kernel", rtol);
}

int wcfd_bicgstab(const wcfd_mesh* m, wcfd_system A, float* x, wcfd_krylov_ws ws, double atol, int32_t maxiter,
                  wcfd_solve_stats* stats, void* stream) {
    return bicgstab_solve(m, A, x, ws, atol, 0.0, maxiter, stats, stream);
}

int wcfd_krylov_solve(const wcfd_mesh* m, wcfd_system A, float* x, wcfd_krylov_ws ws, int32_t method,
                      double atol, double rtol, int32_t maxiter, wcfd_solve_stats* stats, void* stream) {
    RET_IF(method != 0 && method != 1, WCFD_ERR_ARGUMENT, "method must be 0 (cg) or 1 (bicgstab)");
    if (method == 1) return bicgstab_solve(m, A, x, ws, atol, rtol, maxiter, stats, stream);
    return cg_solve(m, A, x, ws, atol, rtol, maxiter, stats, stream);
}

int wcfd_simple_iteration(const wcfd_case* cp, void* stream) {
    RET_IF(!cp, WCFD_ERR_ARGUMENT, "case is null");
    const wcfd_case& c = *cp;
    int rc = check_mesh(&c.mesh);
    if (rc) return rc;
    RET_IF(!c.hbya || !c.p_x || !c.rua || !c.rua_faces || !c.div || !c.stats, WCFD_ERR_ARGUMENT, "null case array");
    RET_IF(c.prm.n_inner < 0 || c.prm.n_ortho < 0, WCFD_ERR_ARGUMENT, "negative loop count");
    cudaStream_t st = S(stream);
    NvtxRange step_range(c.prm.steady ? "wcfd SIMPLE iteration" : "wcfd PISO step");
    const wcfd_mesh& m = c.mesh;
    const uint32_t skew = c.prm.skew ? 4u : 0u;
    const int gc = grid_for(m.n_cells);
    // the face kernels are persistent: resident blocks striding over the faces
    const int gfa = resident_grid((const void*)face_pass_kernel, m.n_faces);
    const int gfp = resident_grid((const void*)face_pass_partial_kernel, m.n_faces);
    const int gfc = resident_grid((const void*)cell_to_face_kernel, m.n_faces);
    // incompressible.py:96-99
    face_pass_kernel<<<gfa, kBlock, 0, st>>>(m, c.bc, c.state, WCFD_ALL, 1u | 2u | skew | (c.prm.rhie_chow ? 16u : 0u),
                                            c.rua_faces);
    LAUNCH_CHECK("face_pass_kernel");
    gradient_kernel<<<gc, kBlock, 0, st>>>(m, c.state, WCFD_ALL, nullptr, CorrectArgs{nullptr, nullptr});
    LAUNCH_CHECK("gradient_kernel");
    // :102-116
    rc = wcfd_assemble_momentum(cp, stream);
    if (rc) return rc;
    auto mark = [&](int i) {
        if (c.events && c.events[i]) cudaEventRecord(reinterpret_cast<cudaEvent_t>(c.events[i]), st);
    };
    mark(0);
    {
        NvtxRange r("wcfd momentum solve");
        rc = bicgstab_solve(&m, c.mom, c.hbya, c.ws_u, c.prm.atol_u, c.prm.rtol_u, c.prm.maxiter, c.stats + 0, stream);
    }
    if (rc) return rc;
    mark(1);
    // :118-123
    hbya_kernel<<<gc, kBlock, 0, st>>>(m.n_cells, c.state.cell_gradients, c.rua, c.hbya, c.state.cell_values);
    LAUNCH_CHECK("hbya_kernel");
    cell_to_face_kernel<<<gfc, kBlock, 0, st>>>(m, c.rua, c.rua_faces);
    LAUNCH_CHECK("cell_to_face_kernel");
    for (int inner = 0; inner < c.prm.n_inner; ++inner) {
        NvtxRange r("wcfd pressure corrector");
        for (int ortho = 0; ortho < c.prm.n_ortho; ++ortho) {
            // :127-132
            face_pass_kernel<<<gfa, kBlock, 0, st>>>(m, c.bc, c.state, WCFD_ALL, 2u | skew, nullptr);
            LAUNCH_CHECK("face_pass_kernel");
            gradient_kernel<<<gc, kBlock, 0, st>>>(m, c.state, WCFD_ALL, c.div, CorrectArgs{nullptr, nullptr});
            LAUNCH_CHECK("gradient_kernel");
            // :134-142
            rc = wcfd_assemble_pressure(cp, stream);
            if (rc) return rc;
            const bool last = inner == c.prm.n_inner - 1 && ortho == c.prm.n_ortho - 1;
            if (last) mark(2);
            if (c.prm.p_refine > 0)
                rc = wcfd_cg_refine(&m, c.pres, c.p_x64, c.p_x, c.p_work, c.ws_p, c.prm.p_refine, c.prm.p_refine_rtol,
                                    c.prm.maxiter, c.stats + 1, stream);
            else
                rc = cg_solve(&m, c.pres, c.p_x, c.ws_p, c.prm.atol_p, c.prm.rtol_p, c.prm.maxiter, c.stats + 1, stream);
            if (rc) return rc;
            if (last) mark(3);
            // :144-147
            p_update_kernel<<<gc, kBlock, 0, st>>>(m.n_cells, c.p_x, c.state.cell_values,
                                                   c.prm.steady ? c.prm.p_relax : 0.0f);
            LAUNCH_CHECK("p_update_kernel");
            // :150-156
            face_pass_partial_kernel<<<gfp, kBlock, 0, st>>>(m, c.bc, c.state, WCFD_P, skew, nullptr);
            LAUNCH_CHECK("face_pass_partial_kernel");
            gradient_kernel<<<gc, kBlock, 0, st>>>(m, c.state, WCFD_P, nullptr, CorrectArgs{c.hbya, c.rua});
            LAUNCH_CHECK("gradient_kernel");
        }
    }
    return WCFD_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------
// Allocation-free CG: the workspace lives in a fixed-size array in the library's own
// device memory instead of coming from the caller.
//
// For callers that own their input and output arrays but cannot create device
// workspace: a host code that drives the pressure solve through this C ABI with a
// device-memory budget fixed at start-up, or a plugin that is not allowed to allocate
// once its host application runs.  The array is a file-scope __device__ variable, so
// every GPU that loads the library holds it (kNoAllocBytes, about 3.1 MiB) until the
// process exits.
//
// The host only knows a stand-in for the array's name; its device address is looked up
// with cudaGetSymbolAddress and then passed to the kernel.  A call made outside stream
// capture looks the address up again (so a device reset, which reloads the module at a
// new address, is picked up) and remembers it per device; a call made while its stream
// is being captured uses the remembered address, so the first call on a device, and the
// first call after a device reset, must come before any capture.  All calls share the
// one array: the call zeroes the barrier words it needs, and calls that overlap on the
// GPU (other streams, other threads) race on it.
namespace {

constexpr size_t kNoAllocVecBytes = 6ull * WCFD_NOALLOC_MAX_CELLS * sizeof(float);
constexpr size_t kNoAllocPartialsOff = (kNoAllocVecBytes + 255) / 256 * 256;
constexpr size_t kNoAllocPartialsBytes = 8ull * WCFD_MAX_BLOCKS * sizeof(double);
constexpr size_t kNoAllocBarrierOff = kNoAllocPartialsOff + kNoAllocPartialsBytes;
constexpr size_t kNoAllocBytes = kNoAllocBarrierOff + WCFD_BARRIER_WORDS * sizeof(uint32_t);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_noalloc_mu;
void* g_noalloc_addr[64] = {nullptr};

}  // namespace

extern "C" int wcfd_cg_noalloc(const wcfd_mesh* m, wcfd_system A, float* x, double atol, int32_t maxiter,
                               wcfd_solve_stats* stats, void* stream) {
    int rc = check_mesh(m);
    if (rc) return rc;
    RET_IF(A.ncomp != 1, WCFD_ERR_ARGUMENT, "cg solves scalar systems (ncomp 1)");
    RET_IF(m->n_cells > WCFD_NOALLOC_MAX_CELLS, WCFD_ERR_TOO_LARGE,
           "wcfd_cg_noalloc: n_cells exceeds WCFD_NOALLOC_MAX_CELLS (use wcfd_cg with a caller workspace)");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return set_error(WCFD_ERR_CUDA, "wcfd_cg_noalloc: no usable current device");
    }
    // a failed query (e.g. the legacy stream while another stream captures in global
    // mode) counts as capturing: only the remembered address is used then
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(S(stream), &cap) != cudaSuccess) {
        cudaGetLastError();
        cap = cudaStreamCaptureStatusActive;
    }
    const bool capturing = cap != cudaStreamCaptureStatusNone;
    void* base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (!capturing || !g_noalloc_addr[dev]) {
            RET_IF(capturing, WCFD_ERR_ARGUMENT,
                   "wcfd_cg_noalloc: the first call on a device must come before any stream capture");
            void* p = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                cudaGetLastError();
                std::snprintf(g_last_error, sizeof(g_last_error), "wcfd_cg_noalloc: cudaGetSymbolAddress: %s",
                              cudaGetErrorString(e));
                return WCFD_ERR_CUDA;
            }
            g_noalloc_addr[dev] = p;
        }
        base = g_noalloc_addr[dev];
    }
    unsigned char* b = static_cast<unsigned char*>(base);
    wcfd_krylov_ws ws;
    ws.vec = reinterpret_cast<float*>(b);
    ws.partials = reinterpret_cast<double*>(b + kNoAllocPartialsOff);
    ws.results = nullptr;
    ws.barrier = reinterpret_cast<uint32_t*>(b + kNoAllocBarrierOff);
    return launch_krylov(cg_kernel_for(m->ell_width, m->ell_dcol != nullptr), 0, m, A, x, ws, atol, maxiter, stats, S(stream), "cg_kernel");
}
