// Field operators of the finite-volume step: boundary values + face interpolation
// (+ mass flux), Green-Gauss gradients (+ divergence of the mass flux), cell -> face
// interpolation.  One thread per face or per cell; no atomics, so every result is
// bit-reproducible.
#include "common.cuh"
#include "kernels.cuh"

namespace wcfd {

// Face pass (warp_cfd: conditions.py:5-19, interpolation_kernels.py:5-54,
// interpolation_functions.py:5-28, skewness_functions.py:6-19, model_kernels.py:45-60).
//   internal face: phi_f = psi phi_P + (1-psi) phi_N
//                          + (psi grad_P + (1-psi) grad_N) . (r_f - (psi r_P + (1-psi) r_N))
//   boundary face: fixed value -> phi_f = value; fixed gradient g -> phi_f = phi_P + |r_Pf| g
//   mass flux:     mdot = (u_f, v_f, w_f) . n_owner * A
// flags: bit0 apply every field's boundary table first (set_boundary_conditions),
//        bit1 recompute the mass flux, bit2 skew correction, bit3 upwind instead of
//        linear interpolation on internal faces (phi_P if mdot > 0 else phi_N,
//        interpolation_functions.py:18-28; used by face_interpolation(upwind=True)),
//        bit4 (opt-in, not the reference's path) Rhie-Chow flux on internal faces:
//        mdot = u_f . n A - rUA_f (gdiff (p_N - p_P) - (psi grad p_P + (1-psi) grad p_N) . n A)
//        with the pressure equation's own compact coefficient gdiff, so the convecting flux is
//        the pressure equation's face flux (the form of FV/_deprecated/mesh_ops.py:59-93,
//        written with the full owner-to-neighbour distance); rua_f may be null otherwise.
// kAll: 1 when the caller knows mask == WCFD_ALL, 0 when it knows it is not (the code for
// the whole-record path is then left out, and with it its registers), -1 to test at run time.
// The face's own records ([K] arrays) do not depend on the cell ids: they are issued
// with the ids, so a face is two global-memory round trips deep (ids and records, then
// the cells).  The persistent kernels below issue the next face's records before the
// current face's cell loads, so the two round trips of consecutive faces overlap.
struct FaceRec {
    int P, N;
    float4 gi, nrm;
};

__device__ __forceinline__ FaceRec load_face_rec(const wcfd_mesh& m, uint32_t flags, int k) {
    FaceRec r;
    r.P = __ldg(m.face_owner + k);
    r.N = __ldg(m.face_nbr + k);
    r.gi = __ldg(reinterpret_cast<const float4*>(m.face_interp) + k);
    r.nrm = (flags & 2u) ? __ldg(reinterpret_cast<const float4*>(m.face_normal) + k)
                         : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    return r;
}

template <int kAll = -1>
__device__ __forceinline__ void face_pass_rec(const wcfd_mesh& m, const wcfd_bc& bc, const wcfd_state& s, uint32_t mask_in, uint32_t flags, int k,
                                              const FaceRec& rec, const float* __restrict__ rua_f = nullptr) {
    const uint32_t mask = kAll == 1 ? (uint32_t)WCFD_ALL : mask_in;
    const bool all = kAll < 0 ? mask == WCFD_ALL : kAll == 1;
    const int P = rec.P;
    const int N = rec.N;
    const float4 gi = rec.gi;
    const float4 nrm = rec.nrm;
    // an internal face with every field selected overwrites all four values: no read
    float4 fv = (N >= 0 && all) ? make_float4(0.0f, 0.0f, 0.0f, 0.0f) : ld4(s.face_values + 4 * (size_t)k);
    const float4 cp = ld4(s.cell_values + 4 * (size_t)P);
    if (N >= 0) {
        const float psi = gi.w;
        const float psi2 = 1.0f - psi;
        const float4 cn = ld4(s.cell_values + 4 * (size_t)N);
        // every field: a cell's 4 x 3 gradients are 48 bytes, three 128-bit loads; a
        // single field: only its three components
        const float* gPp = s.cell_gradients + 12 * (size_t)P;
        const float* gNp = s.cell_gradients + 12 * (size_t)N;
        float gP[12], gN[12];
        if ((flags & 4u) && all) {
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                const float4 a = ld4(gPp + 4 * q);
                const float4 b = ld4(gNp + 4 * q);
                gP[4 * q] = a.x; gP[4 * q + 1] = a.y; gP[4 * q + 2] = a.z; gP[4 * q + 3] = a.w;
                gN[4 * q] = b.x; gN[4 * q + 1] = b.y; gN[4 * q + 2] = b.z; gN[4 * q + 3] = b.w;
            }
        }
#pragma unroll
        for (int o = 0; o < 4; ++o) {
            if (!(mask & (1u << o))) continue;
            float val;
            if (flags & 8u) val = s.mass_fluxes[k] > 0.0f ? comp(cp, o) : comp(cn, o);
            else val = comp(cp, o) * psi + psi2 * comp(cn, o);
            if (flags & 4u) {
                const float px = all ? gP[3 * o] : gPp[3 * o], py = all ? gP[3 * o + 1] : gPp[3 * o + 1];
                const float pz = all ? gP[3 * o + 2] : gPp[3 * o + 2];
                const float nx = all ? gN[3 * o] : gNp[3 * o], ny = all ? gN[3 * o + 1] : gNp[3 * o + 1];
                const float nz = all ? gN[3 * o + 2] : gNp[3 * o + 2];
                const float gx = px * psi + psi2 * nx;
                const float gy = py * psi + psi2 * ny;
                const float gz = pz * psi + psi2 * nz;
                val += gx * gi.x + gy * gi.y + gz * gi.z;
            }
            set_comp(fv, o, val);
        }
    } else {
        const int b = __ldg(m.face_brow + k);
        const uchar4 t = __ldg(reinterpret_cast<const uchar4*>(bc.type) + b);
        const float4 bv = __ldg(reinterpret_cast<const float4*>(bc.value) + b);
        float4 fg = ld4(s.face_gradients + 4 * (size_t)k);
        const uint8_t tt[4] = {t.x, t.y, t.z, t.w};
        if (flags & 1u) {
#pragma unroll
            for (int o = 0; o < 4; ++o) {
                if (tt[o] == 1) set_comp(fv, o, comp(bv, o));
                else if (tt[o] == 2) set_comp(fg, o, comp(bv, o));
            }
            st4(s.face_gradients + 4 * (size_t)k, fg);
        }
        const float rpf = __ldg(m.face_rpf + k);
#pragma unroll
        for (int o = 0; o < 4; ++o) {
            if ((mask & (1u << o)) && tt[o] == 2) set_comp(fv, o, rpf * comp(fg, o) + comp(cp, o));
        }
    }
    st4(s.face_values + 4 * (size_t)k, fv);
    if (flags & 2u) {
        const float4 n = nrm;
        float md = (fv.x * n.x + fv.y * n.y + fv.z * n.z) * n.w;
        if ((flags & 16u) && rua_f && N >= 0) {
            const float psi = gi.w, psi2 = 1.0f - psi;
            const float4 cn = ld4(s.cell_values + 4 * (size_t)N);
            const float* gP = s.cell_gradients + 12 * (size_t)P + 9;
            const float* gN = s.cell_gradients + 12 * (size_t)N + 9;
            const float gn = (gP[0] * psi + psi2 * gN[0]) * n.x + (gP[1] * psi + psi2 * gN[1]) * n.y +
                             (gP[2] * psi + psi2 * gN[2]) * n.z;
            md -= rua_f[k] * (__ldg(m.face_gdiff + k) * (cn.w - cp.w) - gn * n.w);
        }
        s.mass_fluxes[k] = md;
    }
}

template <int kAll = -1>
__device__ __forceinline__ void face_pass_body(const wcfd_mesh& m, const wcfd_bc& bc, const wcfd_state& s, uint32_t mask, uint32_t flags, int k,
                                               const float* __restrict__ rua_f = nullptr) {
    face_pass_rec<kAll>(m, bc, s, mask, flags, k, load_face_rec(m, flags, k), rua_f);
}

// Persistent form: a grid of resident blocks strides over the faces; each thread issues
// the next face's ids and records, then completes the current face.
template <int kAll>
__device__ __forceinline__ void face_pass_loop(const wcfd_mesh& m, const wcfd_bc& bc, const wcfd_state& s, uint32_t mask,
                                               uint32_t flags, const float* rua_f) {
    const int K = m.n_faces;
    const int stride = gridDim.x * kBlock;
    int k = blockIdx.x * kBlock + threadIdx.x;
    if (k >= K) return;
    FaceRec cur = load_face_rec(m, flags, k);
    for (;;) {
        const bool more = k < K - stride;
        FaceRec nxt;
        if (more) nxt = load_face_rec(m, flags, k + stride);
        face_pass_rec<kAll>(m, bc, s, mask, flags, k, cur, rua_f);
        if (!more) break;
        k += stride;
        cur = nxt;
    }
}

// blocks per SM the persistent passes are compiled for (registers: 65,536 / (256 x this)).
// Measured on the 128^3 cavity (field kernels of one SIMPLE iteration): 3 / 5 (the
// all-field pass at 77 registers without spills) 0.777 ms, 4 / 6 (spilling) 0.790 ms,
// 2 / 4 0.799 ms.
#ifndef WCFD_FACE_PASS_MINB
#define WCFD_FACE_PASS_MINB 3
#endif
#ifndef WCFD_FACE_PARTIAL_MINB
#define WCFD_FACE_PARTIAL_MINB 5
#endif

__global__ void __launch_bounds__(kBlock, WCFD_FACE_PASS_MINB) face_pass_kernel(wcfd_mesh m, wcfd_bc bc, wcfd_state s,
                                                           uint32_t mask, uint32_t flags, const float* rua_f) {
    // launched with mask == WCFD_ALL only; the run-time test compiles to faster code here
    // than the compile-time form (measured on the 128^3 cavity: 118.9 against 134.6 us)
    face_pass_loop<-1>(m, bc, s, mask, flags, rua_f);
}

// the same pass for a mask other than WCFD_ALL (the pressure-only pass of the correction
// loop): per-field loads only, fewer registers, more warps in flight
__global__ void __launch_bounds__(kBlock, WCFD_FACE_PARTIAL_MINB) face_pass_partial_kernel(wcfd_mesh m, wcfd_bc bc, wcfd_state s,
                                                                   uint32_t mask, uint32_t flags, const float* rua_f) {
    face_pass_loop<0>(m, bc, s, mask, flags, rua_f);
}

// Green-Gauss gradient (model.py:232-239, model_kernels.py:71-90):
//   grad phi_c = sum_f phi_f A_f n_cf / V_c, gathered per cell in slot order.
// Fields outside `mask` get a zero gradient (the reference zeroes the whole array).
// With `div` != null also div[c] = sum_f (+-) mdot_f (model_kernels.py:26-34).
// With `corr` != null (the pressure correction of incompressible.py:150-156) also
//   HbyA[c] -= rUA[c] grad p ; cell u,v,w = HbyA.
__device__ __forceinline__ void gradient_body(const wcfd_mesh& m, const wcfd_state& s, uint32_t mask, float* __restrict__ div, const CorrectArgs& corr, int c) {
    const int C = m.n_cells;
    float g[4][3];
#pragma unroll
    for (int o = 0; o < 4; ++o) g[o][0] = g[o][1] = g[o][2] = 0.0f;
    float dv = 0.0f;
    const float4* slots = reinterpret_cast<const float4*>(m.cell_slot);
    // every slot record first (independent loads), then the faces: a thread's chain of
    // global-memory round trips is two deep instead of two per face
    float4 sls[kMaxSlots];
#pragma unroll
    for (int f = 0; f < kMaxSlots; ++f)
        sls[f] = f < m.faces_per_cell ? __ldg(slots + (size_t)f * C + c)
                                      : make_float4(0.0f, 0.0f, 0.0f, __int_as_float(kNullSlot));
#pragma unroll
    for (int f = 0; f < kMaxSlots; ++f) {
        // a null slot (mixed meshes, or past faces_per_cell) reads face 0 and adds nothing:
        // its vector is zero and its flux is masked; a select, not a branch
        const float4 sl = sls[f];
        const int sk = __float_as_int(sl.w);
        const bool real = sk != kNullSlot;
        const int k = !real ? 0 : sk >= 0 ? sk : ~sk;
        const float4 fv = ld4(s.face_values + 4 * (size_t)k);
#pragma unroll
        for (int o = 0; o < 4; ++o) {
            if (!(mask & (1u << o))) continue;
            const float phi = comp(fv, o);
            g[o][0] += phi * sl.x;
            g[o][1] += phi * sl.y;
            g[o][2] += phi * sl.z;
        }
        if (div) {
            const float md = s.mass_fluxes[k];
            dv += !real ? 0.0f : sk >= 0 ? md : -md;
        }
    }
    float* gc = s.cell_gradients + 12 * (size_t)c;
    st4(gc + 0, make_float4(g[0][0], g[0][1], g[0][2], g[1][0]));
    st4(gc + 4, make_float4(g[1][1], g[1][2], g[2][0], g[2][1]));
    st4(gc + 8, make_float4(g[2][2], g[3][0], g[3][1], g[3][2]));
    if (div) div[c] = dv;
    if (corr.hbya) {
        const float r = corr.rua[c];
        float* h = corr.hbya + 3 * (size_t)c;
        const float hx = h[0] - g[3][0] * r;
        const float hy = h[1] - g[3][1] * r;
        const float hz = h[2] - g[3][2] * r;
        h[0] = hx; h[1] = hy; h[2] = hz;
        float* cv = s.cell_values + 4 * (size_t)c;
        cv[0] = hx; cv[1] = hy; cv[2] = hz;
    }
}

__global__ void __launch_bounds__(kBlock) gradient_kernel(wcfd_mesh m, wcfd_state s, uint32_t mask,
                                                          float* __restrict__ div, CorrectArgs corr) {
    const int c = blockIdx.x * kBlock + threadIdx.x;
    if (c >= m.n_cells) return;
    gradient_body(m, s, mask, div, corr, c);
}

// mdot = (u_f, v_f, w_f) . n_owner * A (model_kernels.py:45-60)
__device__ __forceinline__ void mass_flux_body(const wcfd_mesh& m, const wcfd_state& s, int k) {
    const float4 fv = ld4(s.face_values + 4 * (size_t)k);
    const float4 n = __ldg(reinterpret_cast<const float4*>(m.face_normal) + k);
    s.mass_fluxes[k] = (fv.x * n.x + fv.y * n.y + fv.z * n.z) * n.w;
}

__global__ void __launch_bounds__(kBlock) mass_flux_kernel(wcfd_mesh m, wcfd_state s) {
    const int k = blockIdx.x * kBlock + threadIdx.x;
    if (k >= m.n_faces) return;
    mass_flux_body(m, s, k);
}

// div[c] = sum over the cell's faces of +mdot (owner side) or -mdot (model_kernels.py:26-34)
__device__ __forceinline__ void div_body(const wcfd_mesh& m, const float* __restrict__ mdot, float* __restrict__ div, int c) {
    const int C = m.n_cells;
    const float4* slots = reinterpret_cast<const float4*>(m.cell_slot);
    float dv = 0.0f;
    for (int f = 0; f < m.faces_per_cell; ++f) {
        const int sk = __float_as_int(__ldg(&slots[(size_t)f * C + c].w));
        const bool real = sk != kNullSlot;
        const float md = mdot[!real ? 0 : sk >= 0 ? sk : ~sk];
        dv += !real ? 0.0f : sk >= 0 ? md : -md;
    }
    div[c] = dv;
}

__global__ void __launch_bounds__(kBlock) div_kernel(wcfd_mesh m, const float* __restrict__ mdot,
                                                     float* __restrict__ div) {
    const int c = blockIdx.x * kBlock + threadIdx.x;
    if (c >= m.n_cells) return;
    div_body(m, mdot, div, c);
}

// interpolate_cell_value_to_face (solver_kernels.py:21-36)
__device__ __forceinline__ void cell_to_face_body(const wcfd_mesh& m, const float* __restrict__ x, float* __restrict__ y, int k) {
    const int P = __ldg(m.face_owner + k);
    const int N = __ldg(m.face_nbr + k);
    if (N < 0) {
        y[k] = x[P];
    } else {
        const float psi = __ldg(m.face_interp + 4 * (size_t)k + 3);
        y[k] = psi * x[P] + (1.0f - psi) * x[N];
    }
}

// persistent, the next face's ids and weight issued before the current face's cell loads
__global__ void __launch_bounds__(kBlock) cell_to_face_kernel(wcfd_mesh m, const float* __restrict__ x,
                                                              float* __restrict__ y) {
    const int K = m.n_faces;
    const int stride = gridDim.x * kBlock;
    int k = blockIdx.x * kBlock + threadIdx.x;
    if (k >= K) return;
    int P = __ldg(m.face_owner + k), N = __ldg(m.face_nbr + k);
    float psi = __ldg(m.face_interp + 4 * (size_t)k + 3);
    for (;;) {
        const bool more = k < K - stride;
        int Pn = 0, Nn = 0;
        float psin = 0.0f;
        if (more) {
            Pn = __ldg(m.face_owner + k + stride);
            Nn = __ldg(m.face_nbr + k + stride);
            psin = __ldg(m.face_interp + 4 * (size_t)(k + stride) + 3);
        }
        y[k] = N < 0 ? x[P] : psi * x[P] + (1.0f - psi) * x[N];
        if (!more) break;
        k += stride;
        P = Pn;
        N = Nn;
        psi = psin;
    }
}

// After the momentum solve (incompressible.py:118-123):
//   HbyA += rUA grad p ; cell u,v,w = HbyA.
// Optionally rUA_f as in cell_to_face for the faces of the same index range.
__device__ __forceinline__ void hbya_body(int C, const float* __restrict__ grad, const float* __restrict__ rua, float* __restrict__ hbya, float* __restrict__ cell_values, int c) {
    const float r = rua[c];
    const float* gp = grad + 12 * (size_t)c + 9;
    float* h = hbya + 3 * (size_t)c;
    const float hx = h[0] + gp[0] * r;
    const float hy = h[1] + gp[1] * r;
    const float hz = h[2] + gp[2] * r;
    h[0] = hx; h[1] = hy; h[2] = hz;
    float* cv = cell_values + 4 * (size_t)c;
    cv[0] = hx; cv[1] = hy; cv[2] = hz;
}

__global__ void __launch_bounds__(kBlock) hbya_kernel(int C, const float* __restrict__ grad,
                                                      const float* __restrict__ rua, float* __restrict__ hbya,
                                                      float* __restrict__ cell_values) {
    const int c = blockIdx.x * kBlock + threadIdx.x;
    if (c >= C) return;
    hbya_body(C, grad, rua, hbya, cell_values, c);
}

// rUA = V / (a_P rho) from the u-row diagonal (solver_kernels.py:6-16), the expression of
// the fused momentum assembly
__global__ void __launch_bounds__(kBlock) rua_kernel(int C, const float* __restrict__ vol, const float* __restrict__ diag3,
                                                     float rho, float* __restrict__ rua) {
    const int c = blockIdx.x * kBlock + threadIdx.x;
    if (c >= C) return;
    rua[c] = vol[c] / (diag3[3 * (size_t)c] * rho);
}

// HbyA += rUA grad p on 3C interleaved rows (solver_kernels.py:38-43), the expression of
// hbya_body
__global__ void __launch_bounds__(kBlock) hbya_add_kernel(int C, const float* __restrict__ pgrad3,
                                                          const float* __restrict__ rua, float* __restrict__ hbya) {
    const int c = blockIdx.x * kBlock + threadIdx.x;
    if (c >= C) return;
    const float r = rua[c];
#pragma unroll
    for (int o = 0; o < 3; ++o) hbya[3 * (size_t)c + o] = hbya[3 * (size_t)c + o] + pgrad3[3 * (size_t)c + o] * r;
}

// p = alpha p_new + (1 - alpha) p (model.py:381-384), or p = p_new (alpha <= 0).
__device__ __forceinline__ void p_update_body(int C, const float* __restrict__ p_new, float* __restrict__ cell_values, float alpha, int c) {
    float* p = cell_values + 4 * (size_t)c + 3;
    if (alpha > 0.0f) *p = alpha * p_new[c] + (1.0f - alpha) * *p;
    else *p = p_new[c];
}

__global__ void __launch_bounds__(kBlock) p_update_kernel(int C, const float* __restrict__ p_new,
                                                          float* __restrict__ cell_values, float alpha) {
    const int c = blockIdx.x * kBlock + threadIdx.x;
    if (c >= C) return;
    p_update_body(C, p_new, cell_values, alpha, c);
}

}  // namespace wcfd

// ---------------------------------------------------------------------------------
// Batched forms: one launch for every case of a device case table; blockIdx.y is the
// case, blockIdx.x runs over that case's faces or cells (blocks past the end of a smaller
// case return at once).  The block size is a launch parameter (autotuned per batch).  The arithmetic is the single-case kernels' (same bodies).
namespace wcfd {

__global__ void __launch_bounds__(kMaxFieldBlock) face_pass_batched(const wcfd_case* __restrict__ cases, uint32_t mask,
                                                            uint32_t flags) {
    const wcfd_case& c = cases[blockIdx.y];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= c.mesh.n_faces) return;
    // the Rhie-Chow option applies to the convecting flux, formed by the pass that also
    // applies the boundary values (the first of an outer iteration)
    const uint32_t rc = (c.prm.rhie_chow && (flags & 1u)) ? 16u : 0u;
    face_pass_body(c.mesh, c.bc, c.state, mask, flags | rc | (c.prm.skew ? 4u : 0u), k, c.rua_faces);
}

// the batched pass for a mask other than WCFD_ALL (the pressure-only pass), compiled
// without the whole-record path like face_pass_partial_kernel
__global__ void __launch_bounds__(kMaxFieldBlock, 3) face_pass_partial_batched(const wcfd_case* __restrict__ cases,
                                                                              uint32_t mask, uint32_t flags) {
    const wcfd_case& c = cases[blockIdx.y];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= c.mesh.n_faces) return;
    const uint32_t rc = (c.prm.rhie_chow && (flags & 1u)) ? 16u : 0u;
    face_pass_body<0>(c.mesh, c.bc, c.state, mask, flags | rc | (c.prm.skew ? 4u : 0u), k, c.rua_faces);
}

// mode 0: gradients only; 1: + divergence into case.div; 2: + velocity correction
__global__ void __launch_bounds__(kMaxFieldBlock) gradient_batched(const wcfd_case* __restrict__ cases, uint32_t mask,
                                                           int mode) {
    const wcfd_case& c = cases[blockIdx.y];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.mesh.n_cells) return;
    const CorrectArgs corr{mode == 2 ? c.hbya : nullptr, c.rua};
    gradient_body(c.mesh, c.state, mask, mode == 1 ? c.div : nullptr, corr, i);
}

__global__ void __launch_bounds__(kMaxFieldBlock) hbya_batched(const wcfd_case* __restrict__ cases) {
    const wcfd_case& c = cases[blockIdx.y];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.mesh.n_cells) return;
    hbya_body(c.mesh.n_cells, c.state.cell_gradients, c.rua, c.hbya, c.state.cell_values, i);
}

__global__ void __launch_bounds__(kMaxFieldBlock) rua_faces_batched(const wcfd_case* __restrict__ cases) {
    const wcfd_case& c = cases[blockIdx.y];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= c.mesh.n_faces) return;
    cell_to_face_body(c.mesh, c.rua, c.rua_faces, k);
}

__global__ void __launch_bounds__(kMaxFieldBlock) p_update_batched(const wcfd_case* __restrict__ cases) {
    const wcfd_case& c = cases[blockIdx.y];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.mesh.n_cells) return;
    p_update_body(c.mesh.n_cells, c.p_x, c.state.cell_values, c.prm.steady ? c.prm.p_relax : 0.0f, i);
}

}  // namespace wcfd
