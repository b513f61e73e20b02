// Cell-parallel assembly of the momentum and pressure systems into the fixed
// per-mesh pattern (diagonal + W slot-major off-diagonals).  Each cell walks its F local
// faces in slot order and writes only its own row, so no atomics are needed (the
// reference adds per-face weights with atomics, equation_kernels.py:52-122).
#include "common.cuh"
#include "kernels.cuh"

namespace wcfd {

// Momentum row of cell c (the reference's rows 3c+o of the interleaved BSR matrix):
//
//   convection, upwind (convection.py:43-91, convectionScheme.py:28-52), scale +1
//     internal face, this cell's side with outward flux F (= +mdot owner, -mdot neighbour):
//       owner:     w_P = mdot if mdot > 0 else 0 ;  w_N = 0 if mdot > 0 else mdot
//       neighbour: w_P = 0 if mdot > 0 else -mdot; w_N = -mdot if mdot > 0 else 0
//     central difference (prm.convection = 1, interpolation 'central difference'):
//       owner:     w_P = psi mdot ; w_N = (1 - psi) mdot
//       neighbour: w_P = -(1 - psi) mdot ; w_N = -psi mdot
//     boundary face: rhs -= mdot_b phi_b                                   (Q7)
//   diffusion, scale -1 (diffusion.py:113-198): internal  w_P = -nu A/d, w_N = +nu A/d
//     boundary fixed value:     diag += nu A/|r_Pf| ; rhs += nu A/|r_Pf| phi_b
//     boundary fixed gradient:  rhs += nu g A
//   ddt (PISO, ddt.py:24-32): diag += V/dt ; rhs += phi_old V/dt
//   explicit -(1/rho) grad p V (grad.py:20-29, incompressible.py:107)
//   implicit relaxation (equation_kernels.py:128-152):
//     rhs += (1-a)/a diag phi ; diag /= a
//   rUA = V / (diag_u rho) (solver_kernels.py:6-16)
// Internal-face explicit weights never reach the RHS in the reference
// (equation_kernels.py:84-101), so by default none are formed here.  Opt-in
// (prm.explicit_terms, not the reference's path), they enter the RHS as the boundary
// ones do (b -= scale w2):
//   convection: w2 = (+mdot owner, -mdot neighbour) E, E the sum of
//     bit0  grad(phi)_f . skew (convection.py:76-78, skewness_functions.py:6-19) and
//     bit1  upwindLinear: grad(phi)_up . (r_f - r_up) (convectionScheme.py:54-88, with the
//           upwind cell's own centroid-to-face vector)
//   bit2  diffusion, non-orthogonal part: w2 = (+owner, -neighbour) nu A grad(phi)_f . n2,
//         n2 = n - d / (n . d) (laplacianScheme.py:39-67)
// with grad(phi)_f = psi grad(phi)_P + (1 - psi) grad(phi)_N; they need face_dvec.
__device__ __forceinline__ void explicit_internal_terms(const wcfd_mesh& m, const wcfd_state& s, int k, bool owner_side,
                                                        float md, float nu, int bits, int field0, int nf, float* b,
                                                        float scale_conv, float scale_diff) {
    const int P = __ldg(m.face_owner + k), N = __ldg(m.face_nbr + k);
    const float4 si = __ldg(reinterpret_cast<const float4*>(m.face_interp) + k);
    const float4 dv = __ldg(reinterpret_cast<const float4*>(m.face_dvec) + k);
    const float4 nn = __ldg(reinterpret_cast<const float4*>(m.face_normal) + k);
    const float psi = si.w, psi2 = 1.0f - psi;
    const float side = owner_side ? 1.0f : -1.0f;
    const float* gP = s.cell_gradients + 12 * (size_t)P;
    const float* gN = s.cell_gradients + 12 * (size_t)N;
    for (int q = 0; q < nf; ++q) {
        const int o = field0 + q;
        const float gx = gP[3 * o] * psi + psi2 * gN[3 * o];
        const float gy = gP[3 * o + 1] * psi + psi2 * gN[3 * o + 1];
        const float gz = gP[3 * o + 2] * psi + psi2 * gN[3 * o + 2];
        if (bits & 3) {
            float e = (bits & 1) ? gx * si.x + gy * si.y + gz * si.z : 0.0f;
            if (bits & 2) {
                const bool up_owner = md > 0.0f;
                const float* gu = up_owner ? gP + 3 * o : gN + 3 * o;
                const float a = up_owner ? psi2 : -psi;  // r_f - r_up = skew + a d
                e += gu[0] * (si.x + a * dv.x) + gu[1] * (si.y + a * dv.y) + gu[2] * (si.z + a * dv.z);
            }
            b[q] -= scale_conv * (side * md * e);
        }
        if (bits & 4) {
            const float nd = nn.x * dv.x + nn.y * dv.y + nn.z * dv.z;
            const float inv = 1.0f / nd;
            const float n2x = nn.x - dv.x * inv, n2y = nn.y - dv.y * inv, n2z = nn.z - dv.z * inv;
            b[q] -= scale_diff * (side * nu * nn.w * (gx * n2x + gy * n2y + gz * n2z));
        }
    }
}

// XT: the opt-in explicit internal terms are compiled in (their code raises the kernel from
// 32 to 48 registers, so the default instantiation leaves it out)
template <bool XT>
__device__ __forceinline__ void momentum_assemble_body(const wcfd_mesh& m, const wcfd_bc& bc, const wcfd_state& s, const wcfd_system& sys, float* __restrict__ rua, const wcfd_params& prm, int c) {
    const int C = m.n_cells;
    const float nu = prm.nu;
    float dsum = 0.0f;
    float dx[3] = {0.0f, 0.0f, 0.0f};
    float b[3] = {0.0f, 0.0f, 0.0f};
    int j = 0;
    const float4* slots = reinterpret_cast<const float4*>(m.cell_slot);
    // Every slot's face reference first, then every face's flux, neighbour and coefficient,
    // all independent loads: a thread's chain of global-memory round trips is two deep
    // instead of two per face (on small meshes this kernel is bound by that latency).
    // Slots past faces_per_cell and null slots read face 0 and are skipped below.
    int sks[kMaxSlots];
#pragma unroll
    for (int f = 0; f < kMaxSlots; ++f)
        sks[f] = f < m.faces_per_cell ? __float_as_int(__ldg(&slots[(size_t)f * C + c].w)) : kNullSlot;
    float mds[kMaxSlots], gds[kMaxSlots];
    int nbs[kMaxSlots];
#pragma unroll
    for (int f = 0; f < kMaxSlots; ++f) {
        const int sk = sks[f];
        const int k = sk == kNullSlot ? 0 : sk >= 0 ? sk : ~sk;
        mds[f] = s.mass_fluxes[k];
        nbs[f] = __ldg(m.face_nbr + k);
        gds[f] = __ldg(m.face_gdiff + k);
    }
#pragma unroll
    for (int f = 0; f < kMaxSlots; ++f) {
        const int sk = sks[f];
        if (sk == kNullSlot) continue;
        const bool owner_side = sk >= 0;
        const int k = owner_side ? sk : ~sk;
        const float md = mds[f];
        const int N = nbs[f];
        if (N >= 0) {
            const float dcoef = nu * gds[f];
            float w0, w1;
            if (prm.convection == 1) {
                // central difference: (psi, 1 - psi) of mdot for the owner, the mirror image
                // of -mdot for the neighbour (convection.py:43-91)
                const float psi = __ldg(m.face_interp + 4 * (size_t)k + 3), psi2 = 1.0f - psi;
                const float mn = -md;
                w0 = owner_side ? psi * md : psi2 * mn;
                w1 = owner_side ? psi2 * md : psi * mn;
            } else if (owner_side) {
                w0 = md > 0.0f ? md : 0.0f;
                w1 = md > 0.0f ? 0.0f : md;
            } else {
                const float mn = -md;
                w0 = md > 0.0f ? 0.0f : mn;
                w1 = md > 0.0f ? mn : 0.0f;
            }
            dsum += w0 + dcoef;
            sys.off[(size_t)j * C + c] = w1 - dcoef;
            ++j;
            if (XT && prm.explicit_terms)
                explicit_internal_terms(m, s, k, owner_side, md, nu, prm.explicit_terms, 0, 3, b, 1.0f, -1.0f);
        } else {
            const int br = __ldg(m.face_brow + k);
            const uchar4 t = __ldg(reinterpret_cast<const uchar4*>(bc.type) + br);
            const float4 fvb = ld4(s.face_values + 4 * (size_t)k);
            const float4 fgb = ld4(s.face_gradients + 4 * (size_t)k);
            const float area = __ldg(m.face_normal + 4 * (size_t)k + 3);
            const float wd = nu * __ldg(m.face_gdiff + k);
            const uint8_t tt[3] = {t.x, t.y, t.z};
#pragma unroll
            for (int o = 0; o < 3; ++o) {
                b[o] -= md * comp(fvb, o);
                if (tt[o] == 2) {
                    b[o] += nu * comp(fgb, o) * area;
                } else {
                    dx[o] += wd;
                    b[o] += wd * comp(fvb, o);
                }
            }
        }
    }
    for (; j < m.ell_width; ++j) sys.off[(size_t)j * C + c] = 0.0f;
    const float V = __ldg(m.cell_volume + c);
    const float4 cv = ld4(s.cell_values + 4 * (size_t)c);
    const float* gp = s.cell_gradients + 12 * (size_t)c + 9;
    const float neg_inv_rho = -(1.0f / prm.rho);
    float d[3];
#pragma unroll
    for (int o = 0; o < 3; ++o) {
        d[o] = dsum + dx[o];
        if (!prm.steady) {
            const float vd = V / prm.dt;
            d[o] += vd;
            b[o] += comp(cv, o) * vd;
        }
        b[o] += (gp[o] * V) * neg_inv_rho;
        if (prm.steady && prm.u_relax > 0.0f) {
            const float a = prm.u_relax;
            b[o] += (1.0f - a) / a * d[o] * comp(cv, o);
            d[o] = d[o] / a;
        }
        sys.diag[3 * (size_t)c + o] = d[o];
        sys.rhs[3 * (size_t)c + o] = b[o];
    }
    rua[c] = V / (d[0] * prm.rho);
}

template <bool XT>
__global__ void __launch_bounds__(kBlock) momentum_assemble_kernel(wcfd_mesh m, wcfd_bc bc, wcfd_state s,
                                                                   wcfd_system sys, float* __restrict__ rua,
                                                                   wcfd_params prm) {
    const int c = blockIdx.x * kBlock + threadIdx.x;
    if (c >= m.n_cells) return;
    momentum_assemble_body<XT>(m, bc, s, sys, rua, prm, c);
}

void launch_momentum_assemble(bool xt, int grid, cudaStream_t st, const wcfd_mesh& m, const wcfd_bc& bc,
                              const wcfd_state& s, const wcfd_system& sys, float* rua, const wcfd_params& prm) {
    if (xt)
        momentum_assemble_kernel<true><<<grid, kBlock, 0, st>>>(m, bc, s, sys, rua, prm);
    else
        momentum_assemble_kernel<false><<<grid, kBlock, 0, st>>>(m, bc, s, sys, rua, prm);
}

// Implicit relaxation of an assembled system on its diagonal (equation_kernels.py:128-152):
// b += (1 - a)/a d phi ; d /= a, phi the cell value of the row's field (fields field0 ..
// field0 + ncomp - 1 of the C x 4 cell values).  The same expression as the relaxation
// inside momentum_assemble_body, so the two routes give the same bits.
__global__ void __launch_bounds__(kBlock) relax_kernel(int C, wcfd_system sys, const float* __restrict__ cell_values,
                                                       int field0, float a) {
    const int c = blockIdx.x * kBlock + threadIdx.x;
    if (c >= C) return;
    for (int o = 0; o < sys.ncomp; ++o) {
        const size_t r = (size_t)sys.ncomp * c + o;
        const float d = sys.diag[r];
        sys.rhs[r] += (1.0f - a) / a * d * cell_values[4 * (size_t)c + field0 + o];
        sys.diag[r] = d / a;
    }
}

// Row `row` of a scalar system becomes the identity with rhs = value
// (equation_kernels.py:155-175); its column is left as it is.
__global__ void replace_row_kernel(int C, int W, wcfd_system sys, int row, float value) {
    const int j = threadIdx.x;
    if (j < W) sys.off[(size_t)j * C + row] = 0.0f;
    if (j == 0) {
        sys.diag[row] = 1.0f;
        sys.rhs[row] = value;
    }
}

// Pressure row of cell c: DiffusionTerm('p', nu = rUA_f), scale +1 (diffusion.py:113-198)
//   internal:          diag -= rUA_f A/d ; off = +rUA_f A/d
//   boundary value:    diag -= rUA_f A/|r_Pf| ; rhs -= rUA_f A/|r_Pf| p_b
//   boundary gradient: rhs -= rUA_f g A
// then rhs += div(HbyA) (incompressible.py:137) and, for the reference cell, the row
// becomes identity with rhs = value (equation_kernels.py:155-175; its column stays).
template <bool XT>
__device__ __forceinline__ void pressure_assemble_body(const wcfd_mesh& m, const wcfd_bc& bc, const wcfd_state& s, const wcfd_system& sys, const float* __restrict__ rua_faces, const float* __restrict__ div, const wcfd_params& prm, int c) {
    const int C = m.n_cells;
    float d = 0.0f, b = 0.0f;
    int j = 0;
    const bool ref = (c == prm.ref_cell);
    const float4* slots = reinterpret_cast<const float4*>(m.cell_slot);
    // the same two-deep load structure as the momentum assembly
    int sks[kMaxSlots];
#pragma unroll
    for (int f = 0; f < kMaxSlots; ++f)
        sks[f] = f < m.faces_per_cell ? __float_as_int(__ldg(&slots[(size_t)f * C + c].w)) : kNullSlot;
    float cfs[kMaxSlots];
    int nbs[kMaxSlots];
#pragma unroll
    for (int f = 0; f < kMaxSlots; ++f) {
        const int sk = sks[f];
        const int k = sk == kNullSlot ? 0 : sk >= 0 ? sk : ~sk;
        nbs[f] = __ldg(m.face_nbr + k);
        cfs[f] = rua_faces[k] * __ldg(m.face_gdiff + k);
    }
#pragma unroll
    for (int f = 0; f < kMaxSlots; ++f) {
        const int sk = sks[f];
        if (sk == kNullSlot) continue;
        const int k = sk >= 0 ? sk : ~sk;
        const int N = nbs[f];
        const float coef = cfs[f];
        if (N >= 0) {
            d -= coef;
            sys.off[(size_t)j * C + c] = ref ? 0.0f : coef;
            ++j;
            if (XT && (prm.explicit_terms & 4))  // opt-in non-orthogonal explicit part (see momentum)
                explicit_internal_terms(m, s, k, sk >= 0, 0.0f, rua_faces[k], 4, 3, 1, &b, 0.0f, 1.0f);
        } else {
            const int br = __ldg(m.face_brow + k);
            const uint8_t t = __ldg(bc.type + 4 * (size_t)br + 3);
            if (t == 2) {
                const float area = __ldg(m.face_normal + 4 * (size_t)k + 3);
                b -= rua_faces[k] * s.face_gradients[4 * (size_t)k + 3] * area;
            } else {
                d -= coef;
                b -= coef * s.face_values[4 * (size_t)k + 3];
            }
        }
    }
    for (; j < m.ell_width; ++j) sys.off[(size_t)j * C + c] = 0.0f;
    b += div[c];
    if (ref) {
        d = 1.0f;
        b = prm.ref_value;
    }
    sys.diag[c] = d;
    sys.rhs[c] = b;
}

template <bool XT>
__global__ void __launch_bounds__(kBlock) pressure_assemble_kernel(wcfd_mesh m, wcfd_bc bc, wcfd_state s,
                                                                   wcfd_system sys,
                                                                   const float* __restrict__ rua_faces,
                                                                   const float* __restrict__ div, wcfd_params prm) {
    const int c = blockIdx.x * kBlock + threadIdx.x;
    if (c >= m.n_cells) return;
    pressure_assemble_body<XT>(m, bc, s, sys, rua_faces, div, prm, c);
}

void launch_pressure_assemble(bool xt, int grid, cudaStream_t st, const wcfd_mesh& m, const wcfd_bc& bc,
                              const wcfd_state& s, const wcfd_system& sys, const float* rua_faces, const float* div,
                              const wcfd_params& prm) {
    if (xt)
        pressure_assemble_kernel<true><<<grid, kBlock, 0, st>>>(m, bc, s, sys, rua_faces, div, prm);
    else
        pressure_assemble_kernel<false><<<grid, kBlock, 0, st>>>(m, bc, s, sys, rua_faces, div, prm);
}

// y = A x on the mesh pattern; NC = 1 (scalar) or 3 (momentum: shared off-diagonals,
// interleaved components).
template <int NC>
__global__ void __launch_bounds__(kBlock) spmv_kernel(wcfd_mesh m, wcfd_system A, const float* __restrict__ x,
                                                      float* __restrict__ y) {
    const int c = blockIdx.x * kBlock + threadIdx.x;
    if (c >= m.n_cells) return;
    const int C = m.n_cells;
    float acc[NC];
#pragma unroll
    for (int o = 0; o < NC; ++o) acc[o] = A.diag[NC * (size_t)c + o] * x[NC * (size_t)c + o];
    for (int j = 0; j < m.ell_width; ++j) {
        const float a = A.off[(size_t)j * C + c];
        const int col = __ldg(m.ell_col + (size_t)j * C + c);
#pragma unroll
        for (int o = 0; o < NC; ++o) acc[o] += a * x[NC * (size_t)col + o];
    }
#pragma unroll
    for (int o = 0; o < NC; ++o) y[NC * (size_t)c + o] = acc[o];
}

void launch_spmv(const wcfd_mesh& m, wcfd_system A, const float* x, float* y, cudaStream_t st) {
    if (A.ncomp == 1)
        spmv_kernel<1><<<grid_for(m.n_cells), kBlock, 0, st>>>(m, A, x, y);
    else
        spmv_kernel<3><<<grid_for(m.n_cells), kBlock, 0, st>>>(m, A, x, y);
}

}  // namespace wcfd

// Batched assembly over a device case table (blockIdx.y = case).
namespace wcfd {

template <bool XT>
__global__ void __launch_bounds__(kMaxFieldBlock) momentum_assemble_batched(const wcfd_case* __restrict__ cases) {
    const wcfd_case& c = cases[blockIdx.y];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.mesh.n_cells) return;
    momentum_assemble_body<XT>(c.mesh, c.bc, c.state, c.mom, c.rua, c.prm, i);
}

template <bool XT>
__global__ void __launch_bounds__(kMaxFieldBlock) pressure_assemble_batched(const wcfd_case* __restrict__ cases) {
    const wcfd_case& c = cases[blockIdx.y];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.mesh.n_cells) return;
    pressure_assemble_body<XT>(c.mesh, c.bc, c.state, c.pres, c.rua_faces, c.div, c.prm, i);
}

void launch_assemble_batched(bool pressure, bool xt, dim3 grid, int block, cudaStream_t st, const wcfd_case* cases) {
    if (pressure) {
        if (xt)
            pressure_assemble_batched<true><<<grid, block, 0, st>>>(cases);
        else
            pressure_assemble_batched<false><<<grid, block, 0, st>>>(cases);
    } else {
        if (xt)
            momentum_assemble_batched<true><<<grid, block, 0, st>>>(cases);
        else
            momentum_assemble_batched<false><<<grid, block, 0, st>>>(cases);
    }
}

}  // namespace wcfd
