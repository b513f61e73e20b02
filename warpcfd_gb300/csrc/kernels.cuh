// Kernel declarations shared between the .cu files of libwcfd.
#pragma once

#include "common.cuh"

namespace wcfd {

struct CorrectArgs {
    float* hbya;        // null = no velocity correction
    const float* rua;
};

__global__ void face_pass_kernel(wcfd_mesh m, wcfd_bc bc, wcfd_state s, uint32_t mask, uint32_t flags,
                                 const float* rua_f);
__global__ void face_pass_partial_kernel(wcfd_mesh m, wcfd_bc bc, wcfd_state s, uint32_t mask, uint32_t flags,
                                 const float* rua_f);
__global__ void gradient_kernel(wcfd_mesh m, wcfd_state s, uint32_t mask, float* div, CorrectArgs corr);
__global__ void mass_flux_kernel(wcfd_mesh m, wcfd_state s);
__global__ void div_kernel(wcfd_mesh m, const float* mdot, float* div);
__global__ void cell_to_face_kernel(wcfd_mesh m, const float* x, float* y);
__global__ void hbya_kernel(int C, const float* grad, const float* rua, float* hbya, float* cell_values);
__global__ void p_update_kernel(int C, const float* p_new, float* cell_values, float alpha);

// assembly launches; xt selects the kernels with the opt-in explicit internal terms
// (wcfd_params.explicit_terms) compiled in
void launch_momentum_assemble(bool xt, int grid, cudaStream_t st, const wcfd_mesh& m, const wcfd_bc& bc,
                              const wcfd_state& s, const wcfd_system& sys, float* rua, const wcfd_params& prm);
void launch_pressure_assemble(bool xt, int grid, cudaStream_t st, const wcfd_mesh& m, const wcfd_bc& bc,
                              const wcfd_state& s, const wcfd_system& sys, const float* rua_faces, const float* div,
                              const wcfd_params& prm);

// Term / Equation API (terms.cu)
struct TermList {
    int count;
    float scale[WCFD_MAX_TERMS];
    int cell_based[WCFD_MAX_TERMS];
    const float* weights[WCFD_MAX_TERMS];
};
__global__ void convection_weights_kernel(wcfd_mesh m, wcfd_state s, wcfd_term_fields tf, int scheme, float* w);
__global__ void diffusion_weights_kernel(wcfd_mesh m, wcfd_bc bc, wcfd_state s, wcfd_term_fields tf, float nu,
                                         const float* nu_faces, int corrected, int bc_mode, float bc_value, float* w);
__global__ void ddt_weights_kernel(wcfd_mesh m, wcfd_state s, wcfd_term_fields tf, float dt, float* w);
__global__ void grad_weights_kernel(wcfd_mesh m, wcfd_state s, int field, float* w);
__global__ void assemble_terms_kernel(wcfd_mesh m, wcfd_system sys, TermList tl);
__global__ void add_rhs_kernel(int64_t n, float* rhs, const float* a, float scale);

// batched forms over a device case table (blockIdx.y = case)
__global__ void face_pass_batched(const wcfd_case* cases, uint32_t mask, uint32_t flags);
__global__ void face_pass_partial_batched(const wcfd_case* cases, uint32_t mask, uint32_t flags);
__global__ void gradient_batched(const wcfd_case* cases, uint32_t mask, int mode);
__global__ void hbya_batched(const wcfd_case* cases);
__global__ void rua_faces_batched(const wcfd_case* cases);
__global__ void p_update_batched(const wcfd_case* cases);
void launch_assemble_batched(bool pressure, bool xt, dim3 grid, int block, cudaStream_t st, const wcfd_case* cases);

// y = A x (NC = A.ncomp), launched from assemble.cu where the kernel template lives
__global__ void relax_kernel(int C, wcfd_system sys, const float* cell_values, int field0, float a);
__global__ void replace_row_kernel(int C, int W, wcfd_system sys, int row, float value);
__global__ void rua_kernel(int C, const float* vol, const float* diag3, float rho, float* rua);
__global__ void hbya_add_kernel(int C, const float* pgrad3, const float* rua, float* hbya);
void launch_spmv(const wcfd_mesh& m, wcfd_system A, const float* x, float* y, cudaStream_t st);

// persistent Krylov kernels (cooperative launch)
struct KrylovArgs {
    wcfd_mesh m;
    wcfd_system A;
    float* x;
    float* ws;            // workspace vectors
    GridCtl g;
    double atol2;
    double rtol2;         // CG only: also stop when ||r||^2 <= rtol2 ||r0||^2 (0 = off)
    int maxiter;
    wcfd_solve_stats* stats;
};
// kernel instantiations for off-diagonal width W (0..6), nullptr otherwise
// delta: read the columns from wcfd_mesh.ell_dcol (int16 offsets from the row)
const void* cg_kernel_for(int W, bool delta);
const void* barrier_check_kernel_ptr();
const void* bicgstab_kernel_for(int W);
const void* cg_cluster_kernel_for(int W, int R);
const void* cg_cluster_batched_for(int W, int R);
const void* bicgstab_cluster_batched_for(int W);
size_t cluster_cg_smem_bytes(int R, int W);
int cluster_cg_max_rows(int W, int optin);
int cluster_cg_rpt(int R);
const void* cg1_cluster_kernel_for(int W, int R);
size_t cluster_cg1_smem_bytes(int R, int W);
// the batched form's single-reduction CG (wcfd_batch_dims.cg_variant = 1), up to 4,096 rows per CTA
const void* cg1m_cluster_batched_for(int W, int R);
size_t cluster_cg1m_smem_bytes(int R, int W);
const void* residual64_kernel_for(int W);
__global__ void refine_update_kernel(int C, double* x64, const float* d, float* x32);
__global__ void refine_count_kernel(wcfd_solve_stats* stats, int* acc, int first, int last);

inline int grid_for(long long n, int bs = kBlock) { return (int)((n + bs - 1) / bs); }

}  // namespace wcfd
