"""Device geometry: the SoA arrays the kernels read, derived once per mesh on the host.

Quantities the reference derives in float32 from its float32 mesh arrays are derived
the same way here, in float32 and in the same order of operations: the centroid
distance d (mesh.py:276), psi (mesh_structs.py:206-209), the skew vector
(skewness_functions.py:15-16, evaluated there per use from the same float32 operands),
|r_P->f| and the diffusion coefficients.  On meshes whose centroids are not exact in
float32 (prisms, jittered nodes, domains far from the origin) the differences of nearby
centroids cancel digits, and deriving these in float64 instead would move the results
away from the reference's by more than its own rounding.  The Green-Gauss slot vectors
are rounded once from float64.  Definitions (warp_cfd/FV/mesh_structs.py:141-251 and the
term kernels):

* psi = |r_P->f| / |r_P - r_N| (mesh_structs.py:206-209); 0 on boundary faces;
* skew = r_f - (psi r_P + (1 - psi) r_N) (skewness_functions.py:6-19);
* face area = the owner's per-slot area (mesh_structs.py:200);
* gdiff = A/|d| on internal faces (laplacianScheme.py:14-34), A |n1|/|d| with the
  non-orthogonal correction (laplacianScheme.py:39-67, n1 = d/(n_f . d)), and A/|r_Pf|
  on boundary faces (diffusion.py:145-146);
* cell slot vector = n_cf A_f / V_c, the Green-Gauss weight (model_kernels.py:83-88);
* a null slot (a cell of a mixed mesh with fewer faces than F) holds NULL_SLOT as its
  face reference and a zero vector; the kernels skip it.

Layout (HBM): per-face arrays are indexed by the reference's face id; per-cell slot data
and the off-diagonal pattern are slot-major ([F][C], [W][C]) so a warp of consecutive
cells reads consecutive addresses.
"""
from __future__ import annotations

import numpy as np


NULL_SLOT = np.int32(-2**31)  # the face reference of a null slot (kNullSlot in the kernels)


def ell_offsets(ell_col):
    """The ELL columns (slot-major, (W, C)) as int16 offsets from their row when every
    |column - row| fits (a structured or bandwidth-ordered numbering), else None: the grid
    Krylov kernels then stream 2 bytes per slot instead of 4 (wcfd_mesh.ell_dcol)."""
    C = ell_col.shape[1]
    if C == 0:
        return None
    d = ell_col.astype(np.int64) - np.arange(C, dtype=np.int64)[None, :]
    return d.astype(np.int16) if int(np.abs(d).max()) <= 32767 else None


def build_geometry(mesh, correction: bool = False) -> dict:
    fp, cp, g = mesh.face_properties, mesh.cell_properties, mesh._geometry64
    f4 = np.float32
    C, F = cp.faces.shape
    K = fp.unique_faces.shape[0]
    P = fp.adjacent_cells[:, 0].astype(np.int64)
    N = fp.adjacent_cells[:, 1].astype(np.int64)
    sP = fp.cell_face_index[:, 0].astype(np.int64)
    cent = g["centroid"].astype(f4)
    area = g["area"][P, sP].astype(f4)
    n_own = g["normal"][P, sP].astype(f4)
    rpf = np.linalg.norm(g["to_face"][P, sP].astype(f4), axis=1)
    internal = N >= 0
    ii = np.nonzero(internal)[0]
    dvec = np.zeros((K, 3), dtype=f4)
    dvec[ii] = fp.distance[ii].astype(f4)
    dmag = np.linalg.norm(dvec, axis=1)
    psi = np.zeros(K, dtype=f4)
    psi[ii] = rpf[ii] / np.linalg.norm(cent[P[ii]] - cent[N[ii]], axis=1)
    psi2 = (f4(1.0) - psi).astype(f4)
    skew = np.zeros((K, 3), dtype=f4)
    skew[ii] = g["face_centroid"][ii].astype(f4) - (cent[P[ii]] * psi[ii, None] + cent[N[ii]] * psi2[ii, None])
    gdiff = area / rpf                                   # boundary value; internal overwritten
    if correction:
        n1 = dvec[ii] * (f4(1.0) / np.sum(n_own[ii] * dvec[ii], axis=1, dtype=f4))[:, None]
        gdiff[ii] = area[ii] * np.linalg.norm(n1, axis=1) / dmag[ii]
    else:
        gdiff[ii] = area[ii] / dmag[ii]
    bids = fp.boundary_face_ids.astype(np.int64)
    brow = -np.ones(K, dtype=np.int32)
    brow[bids] = np.arange(len(bids), dtype=np.int32)

    face_interp = np.zeros((K, 4), dtype=np.float32)
    face_interp[:, :3] = skew
    face_interp[:, 3] = psi
    face_normal = np.zeros((K, 4), dtype=np.float32)
    face_normal[:, :3] = n_own
    face_normal[:, 3] = area
    face_dvec = np.zeros((K, 4), dtype=np.float32)
    face_dvec[:, :3] = dvec

    vol = g["volume"]
    faces = cp.faces.astype(np.int64)
    side = cp.face_side.astype(np.int64)
    real = faces >= 0
    area64 = g["area"][P, sP]
    svec = g["normal"] * area64[np.maximum(faces, 0)][..., None] / vol[:, None, None]   # (C,F,3)
    signed = np.where(side == 0, faces, ~faces).astype(np.int32)
    if not real.all():
        svec[~real] = 0.0
        signed[~real] = NULL_SLOT
    cell_slot = np.zeros((F, C, 4), dtype=np.float32)
    cell_slot[..., :3] = svec.transpose(1, 0, 2)
    cell_slot[..., 3] = np.ascontiguousarray(signed.T).view(np.float32)

    nbr = cp.neighbors.astype(np.int64)
    m = nbr >= 0
    W = int(m.sum(axis=1).max()) if C else 0
    # at least one row: a mesh without internal faces (W = 0, one cell) still hands the
    # kernels a valid array, whose padding row they never read
    ell_col = np.repeat(np.arange(C, dtype=np.int32)[None, :], max(W, 1), axis=0).copy()
    pos = (np.cumsum(m, axis=1) - 1)
    cc, ff = np.nonzero(m)
    ell_col[pos[cc, ff], cc] = nbr[cc, ff]
    ell_dcol = ell_offsets(ell_col) if W > 0 else None

    return dict(
        n_cells=C, n_faces=K, n_bfaces=len(bids), faces_per_cell=F, ell_width=W,
        face_owner=P.astype(np.int32), face_nbr=N.astype(np.int32), face_brow=brow,
        face_interp=face_interp, face_normal=face_normal, face_gdiff=gdiff.astype(np.float32),
        face_rpf=rpf.astype(np.float32), cell_slot=cell_slot, cell_volume=vol.astype(np.float32),
        ell_col=ell_col.astype(np.int32), boundary_face=bids.astype(np.int32), face_dvec=face_dvec,
        ell_dcol=ell_dcol,
    )
