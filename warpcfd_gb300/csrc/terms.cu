// Term weights and generic assembly of the Term/Equation API (warp_cfd/FV/terms/*.py).
//
// The reference's terms fill per-(cell, local face, field) weight arrays and Equation
// adds them into its BSR matrix with atomics (equation_kernels.py:52-122).  Here each
// thread owns one (cell, slot): it reads the slot's face record (the signed face id of
// cell_slot says which side of the face the cell is on) and writes that cell's weights for
// the face, so no two threads touch the same entry and nothing is scattered; the generic
// assembly then walks each cell's slots in order and writes only that cell's row.
//
// Layouts, as the reference's:
//   face-based term weights  [C][F][n][3]: (owner coefficient, neighbour coefficient,
//                            explicit part) of cell c's side of the face in slot f;
//   cell-based (ddt) weights [C][n][2]:    (diagonal, explicit part);
//   explicit (grad) weights  [C*3]:        grad(field)[c][d] * V_c, interleaved.
#include "common.cuh"
#include "kernels.cuh"

namespace wcfd {

namespace {

struct SlotFace {
    int k;        // face id
    bool owner;   // this cell is the face's owner (lower id)
    bool null_;   // a null slot of a mixed mesh
};

__device__ __forceinline__ SlotFace slot_face(const wcfd_mesh& m, int c, int f) {
    const float4* slots = reinterpret_cast<const float4*>(m.cell_slot);
    const int sk = __float_as_int(__ldg(&slots[(size_t)f * m.n_cells + c].w));
    SlotFace s;
    s.null_ = sk == kNullSlot;
    s.owner = sk >= 0;
    s.k = s.null_ ? 0 : (sk >= 0 ? sk : ~sk);
    return s;
}

__device__ __forceinline__ float3 cell_grad(const wcfd_state& s, int c, int field) {
    const float* g = s.cell_gradients + 12 * (size_t)c + 3 * field;
    return make_float3(g[0], g[1], g[2]);
}

}  // namespace

// ConvectionTerm.calculate_weights (convection.py:43-91, convectionScheme.py:3-88).
// scheme 0 upwind, 1 central difference, 2 upwindLinear.  Per face k with flux mdot:
//   boundary face (owner side):  (0, 0, mdot phi_f)
//   internal face: scheme weights (fw0, fw1, fw2) -- upwind (1, 0) if mdot > 0 else (0, 1),
//     central (psi, 1 - psi); fw2 = the skew correction grad(phi)_f . (r_f - r'_f) with
//     grad(phi)_f = psi grad_P + (1 - psi) grad_N of the term's q-th gradient column (the
//     reference passes the term's local index there, convection.py:77), plus for upwindLinear
//     grad(phi)_up . (r_f - r_up) (the upwind cell's own vector; the reference's neighbour
//     branch reads the owner's vector of another slot, which never reaches a matrix:
//     internal explicit weights are dropped by the assembly);
//     owner side (fw0 m, fw1 m, fw2 m), neighbour side (fw1 (-m), fw0 (-m), fw2 (-m)).
__global__ void __launch_bounds__(kBlock) convection_weights_kernel(wcfd_mesh m, wcfd_state s, wcfd_term_fields tf,
                                                                   int scheme, float* __restrict__ w) {
    const int F = m.faces_per_cell, C = m.n_cells, n = tf.n;
    const int idx = blockIdx.x * kBlock + threadIdx.x;
    if (idx >= C * F) return;
    const int c = idx / F, f = idx - c * F;
    float* out = w + (size_t)idx * n * 3;
    const SlotFace sf = slot_face(m, c, f);
    if (sf.null_) {
        for (int q = 0; q < n; ++q) out[3 * q] = out[3 * q + 1] = out[3 * q + 2] = 0.0f;
        return;
    }
    const int k = sf.k;
    const float md = s.mass_fluxes[k];
    const int N = __ldg(m.face_nbr + k);
    if (N < 0) {
        for (int q = 0; q < n; ++q) {
            out[3 * q] = 0.0f;
            out[3 * q + 1] = 0.0f;
            out[3 * q + 2] = md * s.face_values[4 * (size_t)k + tf.index[q]];
        }
        return;
    }
    const int P = __ldg(m.face_owner + k);
    const float4 si = __ldg(reinterpret_cast<const float4*>(m.face_interp) + k);
    const float4 dv = __ldg(reinterpret_cast<const float4*>(m.face_dvec) + k);
    const float psi = si.w, psi2 = 1.0f - psi;
    float fw0, fw1;
    if (scheme == 1) {
        fw0 = psi;
        fw1 = psi2;
    } else {
        fw0 = md > 0.0f ? 1.0f : 0.0f;
        fw1 = md > 0.0f ? 0.0f : 1.0f;
    }
    const float mn = -md;
    for (int q = 0; q < n; ++q) {
        // skew correction with the term's local column q (convection.py:77)
        const float3 gP = cell_grad(s, P, q), gN = cell_grad(s, N, q);
        float fw2 = (gP.x * psi + psi2 * gN.x) * si.x + (gP.y * psi + psi2 * gN.y) * si.y +
                    (gP.z * psi + psi2 * gN.z) * si.z;
        if (scheme == 2) {
            const bool up_owner = md > 0.0f;
            const int g = tf.index[q];
            const float3 gu = cell_grad(s, up_owner ? P : N, g);
            const float a = up_owner ? psi2 : -psi;  // r_f - r_up = skew + a d
            fw2 += gu.x * (si.x + a * dv.x) + gu.y * (si.y + a * dv.y) + gu.z * (si.z + a * dv.z);
        }
        if (sf.owner) {
            out[3 * q] = fw0 * md;
            out[3 * q + 1] = fw1 * md;
            out[3 * q + 2] = fw2 * md;
        } else {
            out[3 * q] = fw1 * mn;
            out[3 * q + 1] = fw0 * mn;
            out[3 * q + 2] = fw2 * mn;
        }
    }
}

// DiffusionTerm.calculate_weights (diffusion.py:113-198, laplacianScheme.py:14-67), viscosity
// nu (nu_faces[k] when not NULL).  Internal face, d = r_N - r_P, weight nu A:
//   plain:      (-1/|d|, 1/|d|, 0)
//   corrected:  n1 = d / (n . d), (-|n1|/|d|, |n1|/|d|, grad(phi)_f . (n - n1))
//   owner side (fw0 w, fw1 w, fw2 w), neighbour side (-fw1 w, -fw0 w, -fw2 w).
// Boundary face (diffusion.py:124-153): fixed gradient g: (0, 0, nu g A); fixed value
// phi_b: (-nu A/|r_Pf|, 0, nu A/|r_Pf| phi_b).  bc_mode 1 (the term's von_neumann or
// dirchlet option, diffusion.py:26-35, both of which build the reference's von Neumann
// kernel): every boundary face (0, 0, nu bc_value A).
__global__ void __launch_bounds__(kBlock) diffusion_weights_kernel(wcfd_mesh m, wcfd_bc bc, wcfd_state s,
                                                                  wcfd_term_fields tf, float nu,
                                                                  const float* __restrict__ nu_faces, int corrected,
                                                                  int bc_mode, float bc_value, float* __restrict__ w) {
    const int F = m.faces_per_cell, C = m.n_cells, n = tf.n;
    const int idx = blockIdx.x * kBlock + threadIdx.x;
    if (idx >= C * F) return;
    const int c = idx / F, f = idx - c * F;
    float* out = w + (size_t)idx * n * 3;
    const SlotFace sf = slot_face(m, c, f);
    if (sf.null_) {
        for (int q = 0; q < n; ++q) out[3 * q] = out[3 * q + 1] = out[3 * q + 2] = 0.0f;
        return;
    }
    const int k = sf.k;
    const float nuk = nu_faces ? nu_faces[k] : nu;
    const float4 nn = __ldg(reinterpret_cast<const float4*>(m.face_normal) + k);
    const float area = nn.w;
    const int N = __ldg(m.face_nbr + k);
    if (N < 0) {
        const int row = __ldg(m.face_brow + k);
        const float rpf = __ldg(m.face_rpf + k);
        for (int q = 0; q < n; ++q) {
            const int g = tf.index[q];
            if (bc_mode == 1) {
                out[3 * q] = 0.0f;
                out[3 * q + 1] = 0.0f;
                out[3 * q + 2] = nuk * bc_value * area;
            } else if (bc.type[4 * (size_t)row + g] == 2) {
                out[3 * q] = 0.0f;
                out[3 * q + 1] = 0.0f;
                out[3 * q + 2] = nuk * s.face_gradients[4 * (size_t)k + g] * area;
            } else {
                const float weight = nuk * area / rpf;
                out[3 * q] = -weight;
                out[3 * q + 1] = 0.0f;
                out[3 * q + 2] = weight * s.face_values[4 * (size_t)k + g];
            }
        }
        return;
    }
    const int P = __ldg(m.face_owner + k);
    const float4 dv = __ldg(reinterpret_cast<const float4*>(m.face_dvec) + k);
    const float dmag = sqrtf(dv.x * dv.x + dv.y * dv.y + dv.z * dv.z);
    const float weight = nuk * area;
    float fw0 = -1.0f / dmag, fw1 = 1.0f / dmag;
    float n2x = 0.0f, n2y = 0.0f, n2z = 0.0f;
    if (corrected) {
        const float inv = 1.0f / (nn.x * dv.x + nn.y * dv.y + nn.z * dv.z);
        const float n1x = dv.x * inv, n1y = dv.y * inv, n1z = dv.z * inv;
        const float n1m = sqrtf(n1x * n1x + n1y * n1y + n1z * n1z);
        fw0 = -1.0f / dmag * n1m;
        fw1 = 1.0f / dmag * n1m;
        n2x = nn.x - n1x;
        n2y = nn.y - n1y;
        n2z = nn.z - n1z;
    }
    const float psi = __ldg(m.face_interp + 4 * (size_t)k + 3), psi2 = 1.0f - psi;
    for (int q = 0; q < n; ++q) {
        float fw2 = 0.0f;
        if (corrected) {
            const int g = tf.index[q];
            const float3 gP = cell_grad(s, P, g), gN = cell_grad(s, N, g);
            fw2 = (psi * gP.x + psi2 * gN.x) * n2x + (psi * gP.y + psi2 * gN.y) * n2y + (psi * gP.z + psi2 * gN.z) * n2z;
        }
        if (sf.owner) {
            out[3 * q] = fw0 * weight;
            out[3 * q + 1] = fw1 * weight;
            out[3 * q + 2] = fw2 * weight;
        } else {
            out[3 * q] = -fw1 * weight;
            out[3 * q + 1] = -fw0 * weight;
            out[3 * q + 2] = -fw2 * weight;
        }
    }
}

// DdtTerm.calculate_weights, backward Euler (ddt.py:24-32): (V/dt, -phi_c V/dt)
__global__ void __launch_bounds__(kBlock) ddt_weights_kernel(wcfd_mesh m, wcfd_state s, wcfd_term_fields tf, float dt,
                                                            float* __restrict__ w) {
    const int i = blockIdx.x * kBlock + threadIdx.x;
    const int n = tf.n;
    if (i >= m.n_cells * n) return;
    const int c = i / n, q = i - c * n;
    const float vddt = __ldg(m.cell_volume + c) / dt;
    w[2 * (size_t)i] = vddt;
    w[2 * (size_t)i + 1] = -s.cell_values[4 * (size_t)c + tf.index[q]] * vddt;
}

// GradTerm.calculate_weights (grad.py:20-29): grad(field)[c][d] V_c at row 3c + d
__global__ void __launch_bounds__(kBlock) grad_weights_kernel(wcfd_mesh m, wcfd_state s, int field,
                                                             float* __restrict__ w) {
    const int i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= 3 * m.n_cells) return;
    const int c = i / 3, d = i - 3 * c;
    w[i] = s.cell_gradients[12 * (size_t)c + 3 * field + d] * __ldg(m.cell_volume + c);
}

// Equation.form_system (equation.py:99-125) over any list of implicit terms, each with its
// assigned scale (terms.py:88-113): for cell c and component o, in term order and each
// term's slots in order --
//   face-based: diagonal += s w[c][f][o][0] over every slot; the off-diagonal entry of the
//     slot's neighbour += s w[c][f][0][1] (internal faces; the off-diagonal storage is
//     shared by the components and every scheme's neighbour coefficient is the same for
//     all fields); rhs -= s w[c][f][o][2] on boundary faces only (internal explicit weights
//     never reach the RHS in the reference, equation_kernels.py:84-101);
//   cell-based: diagonal += s w[c][o][0]; rhs -= s w[c][o][1]
//     (equation_kernels.py:104-122).
// The row starts from zero (Equation.reset, equation.py:202-204).
__global__ void __launch_bounds__(kBlock) assemble_terms_kernel(wcfd_mesh m, wcfd_system sys, TermList tl) {
    const int c = blockIdx.x * kBlock + threadIdx.x;
    const int C = m.n_cells, F = m.faces_per_cell, W = m.ell_width, n = sys.ncomp;
    if (c >= C) return;
    float dg[3] = {0.0f, 0.0f, 0.0f}, b[3] = {0.0f, 0.0f, 0.0f};
    float od[kMaxSlots];
#pragma unroll
    for (int j = 0; j < kMaxSlots; ++j) od[j] = 0.0f;
    for (int t = 0; t < tl.count; ++t) {
        const float sc = tl.scale[t];
        const float* w = tl.weights[t];
        if (tl.cell_based[t]) {
            for (int o = 0; o < n; ++o) {
                dg[o] += sc * w[2 * ((size_t)c * n + o)];
                b[o] -= sc * w[2 * ((size_t)c * n + o) + 1];
            }
            continue;
        }
        int j = 0;
        for (int f = 0; f < F; ++f) {
            const SlotFace sf = slot_face(m, c, f);
            if (sf.null_) continue;
            const float* e = w + ((size_t)c * F + f) * n * 3;
            for (int o = 0; o < n; ++o) dg[o] += sc * e[3 * o];
            if (__ldg(m.face_nbr + sf.k) >= 0) {
                if (j < kMaxSlots) od[j] += sc * e[1];
                ++j;
            } else {
                for (int o = 0; o < n; ++o) b[o] -= sc * e[3 * o + 2];
            }
        }
    }
    for (int o = 0; o < n; ++o) {
        sys.diag[(size_t)n * c + o] = dg[o];
        sys.rhs[(size_t)n * c + o] = b[o];
    }
    for (int j = 0; j < W; ++j) sys.off[(size_t)j * C + c] = od[j];
}

// Equation.add_RHS (equation.py:167-168): rhs += scale arr
__global__ void __launch_bounds__(kBlock) add_rhs_kernel(int64_t n, float* __restrict__ rhs, const float* __restrict__ a,
                                                        float scale) {
    const int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x;
    if (i < n) rhs[i] += a[i] * scale;
}

}  // namespace wcfd
