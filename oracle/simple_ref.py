"""ORACLE (test infrastructure only): numpy restatement of warp_cfd's SIMPLE/PISO step.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use
this module, as the checker or as the timed CPU baseline.  The product
(``warpcfd_gb300``) never imports it.

What it restates, step by step, with the reference file:line of each piece:

* outer loop / PISO loop ........ warp_cfd/FV/implicit_Solvers/incompressible.py:72-172
* boundary values ............... FV/boundary/conditions.py:5-19
* face interpolation + skew ..... FV/interpolation_Schemes/interpolation_kernels.py:5-54,
                                  interpolation_functions.py:5-28, skewness_functions.py:6-19
* Green-Gauss gradient .......... FV/model.py:232-239, FV/kernels/model_kernels.py:71-90
* mass flux / divergence ........ model_kernels.py:26-60
* convection weights ............ FV/terms/convection.py:43-91, Implicit_Schemes/convectionScheme.py:3-52
* diffusion weights ............. FV/terms/diffusion.py:113-198, Implicit_Schemes/laplacianScheme.py:14-67
* ddt / grad terms .............. FV/terms/ddt.py:24-32, FV/terms/grad.py:20-29
* CSR pattern ................... FV/kernels/equation_kernels.py:10-38 (+ row/column sort)
* assembly ...................... FV/terms/equation.py:99-125, equation_kernels.py:52-122
* implicit relaxation ........... equation_kernels.py:128-152
* reference-pressure row ........ equation_kernels.py:155-175
* rUA / HbyA / rUA_f ............ FV/kernels/solver_kernels.py:6-43
* explicit p relaxation ......... FV/model.py:381-384

including the quirks that change numbers: explicit weights of internal faces never
reach the RHS (equation_kernels.py:84-101 loops over boundary faces only; the opt-in
``explicit_internal`` option, not the reference's path, adds them); a p-only
gradient zeroes every field's gradient (model.py:237); rUA uses the relaxed u-row
diagonal for all three components (solver_kernels.py:14-16); term scale is assigned,
not multiplied (terms.py:92-113).

Parity status: PINNED against the reference's own outputs.  The reference runs only on
NVIDIA Warp (warp-lang, not vendored, pinned warp==1.0.4 at requirements.txt:9), which is
not installed on these machines; tests/golden/make_reference_golden.py runs the unmodified
warp_cfd sources on a numpy stand-in for Warp (oracle/warp_stand_in) in float64 with
tightened Krylov solves, and this restatement, fed the reference's own mesh arrays,
reproduces those fields to <= 5e-11 (tests/test_reference_pin.py: steady cavity, channel,
skew-corrected and non-orthogonally corrected jittered cavities, PISO).  The Krylov
arithmetic of the reference (warp.optim.linear cg / bicgstab with the diagonal
preconditioner, warp.sparse SpMV) lives in warp-lang; this file restates the published
preconditioned CG and right-preconditioned BiCGSTAB with an explicit stop test
``||r||_2 <= atol`` checked before every iteration, ``maxiter`` = 500 and atol = 1e-5
(fp32) / 1e-6 (fp64) as at FV/terms/equation.py:35-39, so at the reference's own loose stop
the two may end a solve at different iterations; with the solves tightened they agree.
Also pinned: the mesh pass against a loop restatement (mesh_ref.py) and the reference's
own mesh arrays, the discrete operators against analytic known answers, and the converged
cavity against the Ghia et al. centre-line tables the reference ships
(examples/LDC/*.txt|csv).
"""
from __future__ import annotations

import numpy as np


# --------------------------------------------------------------------------- geometry
def geometry_from_mesh(mesh) -> dict:
    """Reference-style geometry arrays (float64) from a ``Mesh``'s cells_data/faces_data."""
    cp, fp = mesh.cell_properties, mesh.face_properties
    g = mesh._geometry64
    adj = fp.adjacent_cells.astype(np.int64)
    cfi = fp.cell_face_index.astype(np.int64)
    return dict(
        C=int(cp.faces.shape[0]), K=int(fp.unique_faces.shape[0]), F=int(cp.faces.shape[1]),
        cell_faces=cp.faces.astype(np.int64), normal=g["normal"], cell_area=g["area"],
        neighbors=cp.neighbors.astype(np.int64), face_side=cp.face_side.astype(np.int64),
        to_face=g["to_face"], centroid=g["centroid"], volume=g["volume"],
        adjacent=adj, cell_face_index=cfi, is_boundary=fp.is_boundary.astype(np.int64),
        face_centroid=g["face_centroid"],
        distance=fp.distance.astype(np.float64),   # float32 centroid difference (mesh.py:276)
        internal_ids=fp.internal_face_ids.astype(np.int64),
        boundary_ids=fp.boundary_face_ids.astype(np.int64),
        nnz_per_cell=cp.nnz_per_cell.astype(np.int64),
        face_offset_index=cp.face_offset_index.astype(np.int64),
        slot_valid=(cp.faces >= 0),
    )


def geometry_from_reference_arrays(d) -> dict:
    """The same geometry dict from the arrays the reference's own mesh pass produced
    (``Mesh.cell_properties`` / ``face_properties`` before ``finalize``, float32 as
    preprocess/mesh.py computes them), as stored in tests/golden/ref_*.npz under
    ``mesh_cell_*`` / ``mesh_face_*``."""
    f64 = np.float64
    i64 = np.int64
    faces = d["mesh_cell_faces"].astype(i64)
    return dict(
        C=int(faces.shape[0]), K=int(d["mesh_face_unique_faces"].shape[0]), F=int(faces.shape[1]),
        cell_faces=faces, normal=d["mesh_cell_normal"].astype(f64), cell_area=d["mesh_cell_area"].astype(f64),
        neighbors=d["mesh_cell_neighbors"].astype(i64), face_side=d["mesh_cell_face_side"].astype(i64),
        to_face=d["mesh_cell_cell_centroid_to_face_centroid"].astype(f64),
        centroid=d["mesh_cell_centroids"].astype(f64), volume=d["mesh_cell_volumes"].astype(f64),
        adjacent=d["mesh_face_adjacent_cells"].astype(i64), cell_face_index=d["mesh_face_cell_face_index"].astype(i64),
        is_boundary=d["mesh_face_is_boundary"].astype(i64), face_centroid=d["mesh_face_centroid"].astype(f64),
        distance=d["mesh_face_distance"].astype(f64), internal_ids=d["mesh_face_internal_face_ids"].astype(i64),
        boundary_ids=d["mesh_face_boundary_face_ids"].astype(i64), nnz_per_cell=d["mesh_cell_nnz_per_cell"].astype(i64),
        face_offset_index=d["mesh_cell_face_offset_index"].astype(i64), slot_valid=(faces >= 0),
    )


class Geometry:
    """Geometry cast to the working dtype, plus the per-face values init_structs derives.

    face area = owner's per-slot area (mesh_structs.py:200);
    psi = |r_P->f| / |r_P - r_N| (mesh_structs.py:206-209), psi2 = 1 - psi.
    """

    def __init__(self, geo: dict, T):
        self.T = T
        for k, v in geo.items():
            if isinstance(v, np.ndarray) and np.issubdtype(v.dtype, np.floating):
                v = v.astype(T)
            setattr(self, k, v)
        adj, cfi = self.adjacent, self.cell_face_index
        self.P = adj[:, 0]
        self.N = adj[:, 1]
        self.area = self.cell_area[self.P, cfi[:, 0]]
        self.psi = np.zeros(self.K, dtype=T)
        self.psi2 = np.zeros(self.K, dtype=T)
        ii = self.internal_ids
        otf = self.to_face[self.P[ii], cfi[ii, 0]]
        self.psi[ii] = (np.linalg.norm(otf, axis=-1) /
                        np.linalg.norm(self.centroid[self.P[ii]] - self.centroid[self.N[ii]], axis=-1)).astype(T)
        self.psi2[ii] = T(1.0) - self.psi[ii]
        # |r_P->f| per face (owner side)
        self.rpf = np.linalg.norm(self.to_face[self.P, cfi[:, 0]], axis=-1).astype(T)
        self.n_owner = self.normal[self.P, cfi[:, 0]]


# --------------------------------------------------------------------------- Krylov
def _dot(a, b, R):
    return float(np.dot(a.astype(R), b.astype(R)))


def cg(A, b, x, invdiag, atol, maxiter, R=np.float64, rtol=0.0):
    """Jacobi-preconditioned CG; stop when ||r||_2 <= max(atol, rtol ||r_0||_2) (checked
    before each step; the reference passes atol only, rtol is the relative stop of the
    build's refinement sweeps, warpcfd_gb300/csrc/krylov.cu ``thr2``)."""
    T = x.dtype.type
    r = (b - A @ x).astype(T)
    rr = _dot(r, r, R)
    z = (r * invdiag).astype(T)
    rz = _dot(r, z, R)
    p = z.copy()
    k = 0
    atol2 = max(atol * atol, rtol * rtol * rr)
    while k < maxiter and rr > atol2:
        Ap = (A @ p).astype(T)
        pAp = _dot(p, Ap, R)
        if pAp == 0.0:
            break
        alpha = rz / pAp
        x += T(alpha) * p
        r -= T(alpha) * Ap
        rr = _dot(r, r, R)
        z = (r * invdiag).astype(T)
        rz_new = _dot(r, z, R)
        beta = rz_new / rz if rz != 0.0 else 0.0
        rz = rz_new
        p = (z + T(beta) * p).astype(T)
        k += 1
    return k, float(np.sqrt(rr))


def bicgstab(A, b, x, invdiag, atol, maxiter, R=np.float64):
    """Right-preconditioned (Jacobi) BiCGSTAB; stop when ||r||_2 <= atol."""
    T = x.dtype.type
    r = (b - A @ x).astype(T)
    rr = _dot(r, r, R)
    r0 = r.copy()
    rho = _dot(r0, r, R)
    p = r.copy()
    k = 0
    atol2 = atol * atol
    while k < maxiter and rr > atol2:
        y = (p * invdiag).astype(T)
        v = (A @ y).astype(T)
        r0v = _dot(r0, v, R)
        if r0v == 0.0:
            break
        alpha = rho / r0v
        s = (r - T(alpha) * v).astype(T)
        x += T(alpha) * y
        z = (s * invdiag).astype(T)
        t = (A @ z).astype(T)
        tt = _dot(t, t, R)
        ts = _dot(t, s, R)
        omega = ts / tt if tt != 0.0 else 0.0
        x += T(omega) * z
        r = (s - T(omega) * t).astype(T)
        rr = _dot(r, r, R)
        rho_new = _dot(r0, r, R)
        k += 1
        if omega == 0.0 or rho == 0.0:
            break
        beta = (rho_new / rho) * (alpha / omega)
        rho = rho_new
        p = (r + T(beta) * (p - T(omega) * v)).astype(T)
    return k, float(np.sqrt(rr))


def jacobi_inverse(diag):
    T = diag.dtype.type
    out = np.ones_like(diag)
    nz = diag != 0
    out[nz] = (T(1.0) / diag[nz]).astype(T)
    return out


# --------------------------------------------------------------------------- the case
class OracleCase:
    """State and operators of one incompressible case, in dtype ``T`` (fields) with
    Krylov reductions in ``R``.

    bc_type (B,4) uint8: 1 = fixed value, 2 = fixed normal gradient, per boundary face
    (in ``boundary_ids`` order) and field u,v,w,p; bc_value (B,4).
    """

    def __init__(self, geo: dict, bc_type, bc_value, viscosity, density, *, T=np.float64, R=np.float64,
                 reference_cell=None, reference_value=0.0, correction=False, skew_correction=True,
                 atol=None, maxiter=500, rhie_chow=False, explicit_internal=False, conv_scheme="upwind",
                 p_refine=0, p_refine_rtol=1e-3):
        self.g = Geometry(geo, T)
        self.T, self.R = T, R
        g = self.g
        C, K = g.C, g.K
        self.bc_type = np.asarray(bc_type, dtype=np.uint8)
        self.bc_value = np.asarray(bc_value, dtype=T)
        self.mu, self.rho = viscosity, density
        self.ref_cell, self.ref_value = reference_cell, reference_value
        self.correction = correction
        self.skew = skew_correction
        self.rhie_chow = rhie_chow
        self.explicit_internal = explicit_internal
        self.conv_scheme = conv_scheme
        self.atol = atol if atol is not None else (1e-5 if T == np.float32 else 1e-6)
        self.maxiter = maxiter
        # precision form (not the reference's path): fp64 iterative refinement of the
        # pressure solve, ``p_refine`` sweeps with a relative stop of ``p_refine_rtol`` each
        self.p_refine = int(p_refine)
        self.p_refine_rtol = float(p_refine_rtol)
        self.p_x64 = None
        self.cell_values = np.zeros((C, 4), dtype=T)
        self.cell_gradients = np.zeros((C, 4, 3), dtype=T)
        self.face_values = np.zeros((K, 4), dtype=T)
        self.face_gradients = np.zeros((K, 4), dtype=T)
        self.mass_fluxes = np.zeros(K, dtype=T)
        self.HbyA = np.zeros(3 * C, dtype=T)
        self.p_x = np.zeros(C, dtype=T)
        self.rUA = np.zeros(C, dtype=T)
        self.rUA_faces = np.zeros(K, dtype=T)
        self.log = []
        self._build_pattern()

    # ---- CSR pattern (equation_kernels.py:10-38, then sorted as bsr_from_triplets does)
    def _build_pattern(self):
        g = self.g
        C = g.C
        rows = [np.arange(C)]
        cols = [np.arange(C)]
        m = g.neighbors != -1
        cc, ff = np.nonzero(m)
        rows.append(cc)
        cols.append(g.neighbors[cc, ff])
        r = np.concatenate(rows)
        c = np.concatenate(cols)
        order = np.lexsort((c, r))
        self.pat_rows, self.pat_cols = r[order], c[order]
        self.indptr = np.concatenate([[0], np.cumsum(np.bincount(self.pat_rows, minlength=C))])
        # the slot of a nnz: first local face whose neighbour is the column (get_face_idx,
        # equation_kernels.py:43-49); -1 on the diagonal
        slot = -np.ones(len(r), dtype=np.int64)
        off = self.pat_rows != self.pat_cols
        nb = g.neighbors[self.pat_rows[off]]                      # (n,F)
        hit = nb == self.pat_cols[off][:, None]
        slot[off] = np.argmax(hit, axis=1)
        self.pat_slot = slot
        self.diag_pos = np.nonzero(~off)[0]

    # ---- BC + interpolation + gradients + flux --------------------------------------
    def apply_bc(self):
        """conditions.py:5-19."""
        b = self.g.boundary_ids
        t = self.bc_type
        fixed = t == 1
        grad = t == 2
        fv = self.face_values[b]
        fg = self.face_gradients[b]
        fv[fixed] = self.bc_value[fixed]
        fg[grad] = self.bc_value[grad]
        self.face_values[b] = fv
        self.face_gradients[b] = fg

    def face_interpolation(self, out=(0, 1, 2, 3)):
        """interpolation_kernels.py:5-54 (linear + skew correction; Neumann extrapolation)."""
        g, T = self.g, self.T
        ii = g.internal_ids
        P, N = g.P[ii], g.N[ii]
        psi, psi2 = g.psi[ii], g.psi2[ii]
        if self.skew:
            rk_dash = g.centroid[P] * psi[:, None] + g.centroid[N] * psi2[:, None]
            d = g.face_centroid[ii] - rk_dash
        for o in out:
            val = self.cell_values[P, o] * psi + psi2 * self.cell_values[N, o]
            if self.skew:
                gi = self.cell_gradients[P, o] * psi[:, None] + psi2[:, None] * self.cell_gradients[N, o]
                val = val + np.sum(gi * d, axis=1, dtype=T)
            self.face_values[ii, o] = val
        b = g.boundary_ids
        Pb = g.P[b]
        dist = g.rpf[b]
        for o in out:
            neu = self.bc_type[:, o] == 2
            self.face_values[b[neu], o] = dist[neu] * self.face_gradients[b[neu], o] + self.cell_values[Pb[neu], o]

    def calculate_gradients(self, out=(0, 1, 2, 3)):
        """model.py:232-239: zero every field's gradient, then Green-Gauss for ``out``."""
        g = self.g
        self.cell_gradients[...] = 0
        # null slots of mixed meshes (face id -1) have zero normals; mask them anyway
        area = np.where(g.slot_valid, g.area[g.cell_faces], 0).astype(self.T)   # (C,F)
        for o in out:
            phi = np.where(g.slot_valid, self.face_values[g.cell_faces, o], 0).astype(self.T)  # (C,F)
            vec = (phi * area)[..., None] * g.normal / g.volume[:, None, None]
            acc = np.zeros((g.C, 3), dtype=self.T)
            for f in range(g.F):
                acc += vec[:, f]
            self.cell_gradients[:, o] = acc

    def calculate_mass_flux(self):
        """model_kernels.py:45-60: mdot = (u_f . n_owner) A_f."""
        g = self.g
        v = self.face_values[:, 0:3]
        self.mass_fluxes[:] = np.sum(v * g.n_owner, axis=1, dtype=self.T) * g.area

    def rhie_chow_flux(self, grad_p):
        """Opt-in Rhie-Chow convecting flux (not the reference's path; the form of
        FV/_deprecated/mesh_ops.py:59-93 with the full owner-to-neighbour distance):
        mdot -= rUA_f (c_f (p_N - p_P) - (psi grad p_P + (1-psi) grad p_N) . n A) on internal
        faces, c_f the pressure equation's compact coefficient (A/|d|, x|n1| when corrected),
        grad p the cell gradients as they stand before this iteration's gradient pass."""
        g, T = self.g, self.T
        ii = g.internal_ids
        P, N = g.P[ii], g.N[ii]
        dvec = g.distance[ii]
        dmag = np.linalg.norm(dvec, axis=1).astype(T)
        coef = (g.area[ii] / dmag).astype(T)
        if self.correction:
            nf = g.n_owner[ii]
            n1 = dvec * (T(1.0) / np.sum(nf * dvec, axis=1, dtype=T))[:, None]
            coef = (coef * np.linalg.norm(n1, axis=1).astype(T)).astype(T)
        gf = grad_p[P] * g.psi[ii, None] + g.psi2[ii, None] * grad_p[N]
        gn = np.sum(gf * g.n_owner[ii], axis=1, dtype=T)
        p = self.cell_values[:, 3]
        self.mass_fluxes[ii] -= self.rUA_faces[ii] * (coef * (p[N] - p[P]) - gn * g.area[ii])

    def div_flux(self):
        """model_kernels.py:26-34."""
        g = self.g
        m = np.where(g.slot_valid, self.mass_fluxes[g.cell_faces], 0).astype(self.T)
        sgn = np.where(g.face_side == 0, m, -m)
        acc = np.zeros(g.C, dtype=self.T)
        for f in range(g.F):
            acc += sgn[:, f]
        return acc

    # ---- term weights -----------------------------------------------------------------
    def convection_weights(self, fields=(0, 1, 2), scheme=None):
        """convection.py:43-91 -> (C,F,n,3) [owner, neighbour, explicit].  upwindLinear
        (convectionScheme.py:54-88) adds grad(phi)_up . (r_f - r_up) to the explicit weight,
        with the upwind cell's own centroid-to-face vector (the reference's neighbour branch
        reads the owner's, Q12)."""
        g, T = self.g, self.T
        scheme = self.conv_scheme if scheme is None else scheme
        n = len(fields)
        w = np.zeros((g.C, g.F, n, 3), dtype=T)
        b = g.boundary_ids
        for j, o in enumerate(fields):
            w[g.P[b], g.cell_face_index[b, 0], j, 2] = self.mass_fluxes[b] * self.face_values[b, o]
        ii = g.internal_ids
        m = self.mass_fluxes[ii]
        if scheme in ("upwind", "upwindLinear"):
            fw0 = np.where(m > 0, T(1.0), T(0.0)).astype(T)
            fw1 = np.where(m > 0, T(0.0), T(1.0)).astype(T)
        elif scheme == "central difference":
            fw0, fw1 = g.psi[ii], g.psi2[ii]
        else:
            raise NotImplementedError(scheme)
        P, N = g.P[ii], g.N[ii]
        sP, sN = g.cell_face_index[ii, 0], g.cell_face_index[ii, 1]
        if self.skew:
            rk_dash = g.centroid[P] * g.psi[ii][:, None] + g.centroid[N] * g.psi2[ii][:, None]
            d = g.face_centroid[ii] - rk_dash
        for j, o in enumerate(fields):
            fw2 = np.zeros_like(m)
            if self.skew:  # computed as the reference does; reaches the RHS only opt-in (Q1)
                gi = (self.cell_gradients[P, j] * g.psi[ii][:, None] + g.psi2[ii][:, None] * self.cell_gradients[N, j])
                fw2 = np.sum(gi * d, axis=1, dtype=T)
            if scheme == "upwindLinear":
                up = np.where(m > 0, P, N)
                rvec = (g.face_centroid[ii] - g.centroid[up]).astype(T)
                fw2 = (fw2 + np.sum(self.cell_gradients[up, j] * rvec, axis=1, dtype=T)).astype(T)
            w[P, sP, j, 0] = fw0 * m
            w[P, sP, j, 1] = fw1 * m
            w[P, sP, j, 2] = fw2 * m
            mn = -m
            w[N, sN, j, 0] = fw1 * mn
            w[N, sN, j, 1] = fw0 * mn
            w[N, sN, j, 2] = fw2 * mn
        return w

    def diffusion_weights(self, fields, nu):
        """diffusion.py:113-198 (scalar or per-face nu; plain or |n1|-corrected)."""
        g, T = self.g, self.T
        n = len(fields)
        w = np.zeros((g.C, g.F, n, 3), dtype=T)
        nu_f = (np.full(g.K, T(nu), dtype=T) if np.isscalar(nu) else np.asarray(nu, dtype=T))
        b = g.boundary_ids
        Pb, sb = g.P[b], g.cell_face_index[b, 0]
        for j, o in enumerate(fields):
            neu = self.bc_type[:, o] == 2
            wneu = nu_f[b] * self.face_gradients[b, o] * g.area[b]
            weight = nu_f[b] * g.area[b] / g.rpf[b]
            w[Pb, sb, j, 0] = np.where(neu, T(0.0), -weight)
            w[Pb, sb, j, 1] = T(0.0)
            w[Pb, sb, j, 2] = np.where(neu, wneu, weight * self.face_values[b, o])
        ii = g.internal_ids
        P, N = g.P[ii], g.N[ii]
        sP, sN = g.cell_face_index[ii, 0], g.cell_face_index[ii, 1]
        weight = nu_f[ii] * g.area[ii]
        dvec = g.distance[ii]
        dmag = np.linalg.norm(dvec, axis=1).astype(T)
        for j, o in enumerate(fields):
            if not self.correction:
                fw0 = (T(-1.0) / dmag).astype(T)
                fw1 = (T(1.0) / dmag).astype(T)
                fw2 = np.zeros_like(dmag)
            else:
                nf = g.n_owner[ii]
                n1 = dvec * (T(1.0) / np.sum(nf * dvec, axis=1, dtype=T))[:, None]
                n1m = np.linalg.norm(n1, axis=1).astype(T)
                n2 = nf - n1
                fw0 = (T(-1.0) / dmag * n1m).astype(T)
                fw1 = (T(1.0) / dmag * n1m).astype(T)
                gf = g.psi[ii][:, None] * self.cell_gradients[P, o] + g.psi2[ii][:, None] * self.cell_gradients[N, o]
                fw2 = np.sum(gf * n2, axis=1, dtype=T)
            w[P, sP, j, 0] = fw0 * weight
            w[P, sP, j, 1] = fw1 * weight
            w[P, sP, j, 2] = fw2 * weight
            w[N, sN, j, 0] = -fw1 * weight
            w[N, sN, j, 1] = -fw0 * weight
            w[N, sN, j, 2] = -fw2 * weight
        return w

    def ddt_weights(self, dt, fields=(0, 1, 2)):
        """ddt.py:24-32 -> (C,n,2) [diagonal, explicit]."""
        g, T = self.g, self.T
        vd = (g.volume / T(dt)).astype(T)
        w = np.zeros((g.C, len(fields), 2), dtype=T)
        for j, o in enumerate(fields):
            w[:, j, 0] = vd
            w[:, j, 1] = -self.cell_values[:, o] * vd
        return w

    def grad_term(self, field=3):
        """grad.py:20-29 -> (3C,) grad(p) * V, interleaved."""
        g = self.g
        return (self.cell_gradients[:, field, :] * g.volume[:, None]).astype(self.T).reshape(-1)

    # ---- assembly ---------------------------------------------------------------------
    def assemble(self, n, face_terms, cell_terms=(), explicit=None):
        """equation.py:99-125: returns per-component CSR values (n, nnz) and rhs (C,n).

        face_terms: [(weights (C,F,n,3), scale)]; cell_terms: [(weights (C,n,2), scale)];
        explicit: [(array (n*C,), scale)].
        """
        g, T = self.g, self.T
        nnz = len(self.pat_rows)
        vals = np.zeros((n, nnz), dtype=T)
        rhs = np.zeros((g.C, n), dtype=T)
        diag_rows = self.pat_rows[self.diag_pos]
        off = self.pat_slot >= 0
        for w, s in face_terms:
            s = T(s)
            for o in range(n):
                acc = np.zeros(g.C, dtype=T)
                for f in range(g.F):
                    acc += s * w[:, f, o, 0]
                vals[o, self.diag_pos] += acc[diag_rows]
                vals[o, off] += s * w[self.pat_rows[off], self.pat_slot[off], o, 1]
            b = g.boundary_ids
            for o in range(n):
                np.add.at(rhs[:, o], g.P[b], -s * w[g.P[b], g.cell_face_index[b, 0], o, 2])
            if self.explicit_internal:
                # opt-in (not the reference's path, Q1): internal explicit weights reach the
                # RHS the way the boundary ones do
                ii = g.internal_ids
                for o in range(n):
                    np.add.at(rhs[:, o], g.P[ii], -s * w[g.P[ii], g.cell_face_index[ii, 0], o, 2])
                    np.add.at(rhs[:, o], g.N[ii], -s * w[g.N[ii], g.cell_face_index[ii, 1], o, 2])
        for w, s in cell_terms:
            s = T(s)
            for o in range(n):
                vals[o, self.diag_pos] += (s * w[:, o, 0])[diag_rows]
                rhs[:, o] -= s * w[:, o, 1]
        if explicit is not None:
            for arr, s in explicit:
                rhs += (arr * T(s)).reshape(g.C, n)
        return vals, rhs

    def relax(self, vals, rhs, alpha, fields):
        """equation_kernels.py:128-152 (diagonal entries only)."""
        T = self.T
        a = T(alpha)
        diag_rows = self.pat_rows[self.diag_pos]
        for o, gi in enumerate(fields):
            d = vals[o, self.diag_pos]
            rhs[diag_rows, o] += (T(1.0) - a) / a * d * self.cell_values[diag_rows, gi]
            vals[o, self.diag_pos] = d / a

    def matrix(self, vals_o):
        import scipy.sparse as sp
        return sp.csr_matrix((vals_o, self.pat_cols, self.indptr), shape=(self.g.C, self.g.C))

    def momentum_matrix(self, vals):
        """The interleaved 3C x 3C matrix (row 3c+o), as the reference stores it."""
        import scipy.sparse as sp
        C = self.g.C
        rows = np.concatenate([3 * self.pat_rows + o for o in range(3)])
        cols = np.concatenate([3 * self.pat_cols + o for o in range(3)])
        v = np.concatenate([vals[o] for o in range(3)])
        return sp.csr_matrix((v, (rows, cols)), shape=(3 * C, 3 * C))

    def refined_pressure_solve(self, A, b, invdiag):
        """The build's precision form of the pressure solve (warpcfd_gb300/csrc/capi.cu
        ``wcfd_cg_refine``), not a reference step: ``p_refine`` sweeps of r = b - A x64 in
        fp64 rounded once to the field type, a CG correction solve from zero to
        ||r_k|| <= p_refine_rtol ||r||, x64 += d; the field solution is x64 rounded.  x64
        persists across solves (started from the field solution on first use).  Returns
        the total correction iterations and the fp64 residual norm of the result."""
        T = self.T
        if self.p_x64 is None:
            self.p_x64 = self.p_x.astype(np.float64)
        A64 = A.astype(np.float64)
        b64 = b.astype(np.float64)
        total = 0
        for _ in range(self.p_refine):
            r = (b64 - A64 @ self.p_x64).astype(T)
            d = np.zeros_like(self.p_x)
            k, _ = cg(A, r, d, invdiag, 0.0, self.maxiter, self.R, rtol=self.p_refine_rtol)
            total += k
            self.p_x64 += d.astype(np.float64)
        self.p_x[:] = self.p_x64.astype(T)
        return total, float(np.linalg.norm(b64 - A64 @ self.p_x64))

    # ---- one outer iteration / time step ----------------------------------------------
    def run(self, u_relax=0.7, p_relax=0.3, n_outer=1, n_inner=1, n_ortho=1, steady=True,
            n_time=1, dt=1.0, log=False):
        """incompressible.py:72-172."""
        T = self.T
        g = self.g
        nu = self.mu / self.rho
        inv_rho = 1.0 / self.rho
        for nt in range(n_time if not steady else 1):
            for it in range(n_outer):
                self.apply_bc()
                self.face_interpolation()
                grad_p_prev = self.cell_gradients[:, 3, :].copy()
                self.calculate_gradients()
                self.calculate_mass_flux()
                if self.rhie_chow:
                    self.rhie_chow_flux(grad_p_prev)
                wc = self.convection_weights()
                wd = self.diffusion_weights((0, 1, 2), nu)
                gp = self.grad_term()
                cell_terms = ()
                if not steady:
                    cell_terms = ((self.ddt_weights(dt), 1.0),)
                vals, rhs = self.assemble(3, [(wc, 1.0), (wd, -1.0)], cell_terms, [(gp, -inv_rho)])
                if steady and u_relax is not None:
                    self.relax(vals, rhs, u_relax, (0, 1, 2))
                Ap = vals[:, self.diag_pos]                         # (3,C)
                A = self.momentum_matrix(vals)
                invd = jacobi_inverse(Ap.T.reshape(-1).copy())
                ku, ru = bicgstab(A, rhs.reshape(-1), self.HbyA, invd, self.atol, self.maxiter, self.R)
                p_grad = self.cell_gradients[:, 3, :].reshape(-1).copy()
                self.rUA[:] = (g.volume / (Ap[0] * T(self.rho))).astype(T)      # solver_kernels.py:6-16
                self.HbyA += (p_grad.reshape(-1, 3) * self.rUA[:, None]).reshape(-1)  # :38-43
                ii, b = g.internal_ids, g.boundary_ids                          # :21-36
                self.rUA_faces[b] = self.rUA[g.P[b]]
                self.rUA_faces[ii] = g.psi[ii] * self.rUA[g.P[ii]] + g.psi2[ii] * self.rUA[g.N[ii]]
                self.cell_values[:, 0:3] = self.HbyA.reshape(-1, 3)
                kp = 0
                for _ in range(n_inner):
                    for _ in range(n_ortho):
                        self.face_interpolation()
                        self.calculate_gradients()
                        self.calculate_mass_flux()
                        div = self.div_flux()
                        wpd = self.diffusion_weights((3,), self.rUA_faces)
                        pv, prhs = self.assemble(1, [(wpd, 1.0)])
                        prhs[:, 0] += div
                        if self.ref_cell is not None:                          # equation_kernels.py:155-175
                            rc = self.ref_cell
                            s, e = self.indptr[rc], self.indptr[rc + 1]
                            pv[0, s:e] = np.where(self.pat_cols[s:e] == rc, T(1.0), T(0.0))
                            prhs[rc, 0] = T(self.ref_value)
                        Apm = self.matrix(pv[0])
                        invp = jacobi_inverse(pv[0, self.diag_pos].copy())
                        if self.p_refine > 0:
                            kp, rp = self.refined_pressure_solve(Apm, prhs[:, 0].copy(), invp)
                        else:
                            kp, rp = cg(Apm, prhs[:, 0].copy(), self.p_x, invp, self.atol, self.maxiter, self.R)
                        if steady and p_relax is not None:
                            a = T(p_relax)
                            self.cell_values[:, 3] = a * self.p_x + (T(1.0) - a) * self.cell_values[:, 3]
                        else:
                            self.cell_values[:, 3] = self.p_x
                        self.face_interpolation((3,))
                        self.calculate_gradients((3,))
                        vc = (self.cell_gradients[:, 3, :] * self.rUA[:, None]).reshape(-1)
                        self.HbyA -= vc
                        self.cell_values[:, 0:3] = self.HbyA.reshape(-1, 3)
                if log:
                    self.log.append((ku, ru, kp))
        return self
