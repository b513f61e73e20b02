"""Device geometry: the SoA arrays the kernels read, derived once per mesh on the host.

All derived quantities are computed in float64 from the mesh pass and rounded once to
float32.  Their definitions follow the reference's struct initialisation
(warp_cfd/FV/mesh_structs.py:141-251) and term kernels:

* psi = |r_P->f| / |r_P - r_N| (mesh_structs.py:206-209); 0 on boundary faces;
* skew = r_f - (psi r_P + (1 - psi) r_N) (skewness_functions.py:6-19);
* face area = the owner's per-slot area (mesh_structs.py:200);
* gdiff = A/|d| on internal faces (laplacianScheme.py:14-34), A |n1|/|d| with the
  non-orthogonal correction (laplacianScheme.py:39-67, n1 = d/(n_f . d)), and A/|r_Pf|
  on boundary faces (diffusion.py:145-146);
* cell slot vector = n_cf A_f / V_c, the Green-Gauss weight (model_kernels.py:83-88).

Layout (HBM): per-face arrays are indexed by the reference's face id; per-cell slot data
and the off-diagonal pattern are slot-major ([F][C], [W][C]) so a warp of consecutive
cells reads consecutive addresses.
"""
from __future__ import annotations

import numpy as np


def build_geometry(mesh, correction: bool = False) -> dict:
    fp, cp, g = mesh.face_properties, mesh.cell_properties, mesh._geometry64
    C, F = cp.faces.shape
    K = fp.unique_faces.shape[0]
    P = fp.adjacent_cells[:, 0].astype(np.int64)
    N = fp.adjacent_cells[:, 1].astype(np.int64)
    sP = fp.cell_face_index[:, 0].astype(np.int64)
    cent = g["centroid"]
    area = g["area"][P, sP]
    n_own = g["normal"][P, sP]
    rpf = np.linalg.norm(g["to_face"][P, sP], axis=1)
    internal = N >= 0
    ii = np.nonzero(internal)[0]
    dvec = np.zeros((K, 3))
    dvec[ii] = cent[N[ii]] - cent[P[ii]]
    dmag = np.linalg.norm(dvec, axis=1)
    psi = np.zeros(K)
    psi[ii] = rpf[ii] / dmag[ii]
    skew = np.zeros((K, 3))
    skew[ii] = g["face_centroid"][ii] - (psi[ii, None] * cent[P[ii]] + (1.0 - psi[ii, None]) * cent[N[ii]])
    gdiff = area / rpf                                   # boundary value; internal overwritten
    if correction:
        n1 = dvec[ii] / np.sum(n_own[ii] * dvec[ii], axis=1)[:, None]
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
    svec = g["normal"] * area[faces][..., None] / vol[:, None, None]   # (C,F,3)
    signed = np.where(side == 0, faces, ~faces).astype(np.int32)
    cell_slot = np.zeros((F, C, 4), dtype=np.float32)
    cell_slot[..., :3] = svec.transpose(1, 0, 2)
    cell_slot[..., 3] = np.ascontiguousarray(signed.T).view(np.float32)

    nbr = cp.neighbors.astype(np.int64)
    m = nbr >= 0
    W = int(m.sum(axis=1).max()) if C else 0
    ell_col = np.repeat(np.arange(C, dtype=np.int32)[None, :], max(W, 1), axis=0)[:W].copy()
    pos = (np.cumsum(m, axis=1) - 1)
    cc, ff = np.nonzero(m)
    ell_col[pos[cc, ff], cc] = nbr[cc, ff]

    return dict(
        n_cells=C, n_faces=K, n_bfaces=len(bids), faces_per_cell=F, ell_width=W,
        face_owner=P.astype(np.int32), face_nbr=N.astype(np.int32), face_brow=brow,
        face_interp=face_interp, face_normal=face_normal, face_gdiff=gdiff.astype(np.float32),
        face_rpf=rpf.astype(np.float32), cell_slot=cell_slot, cell_volume=vol.astype(np.float32),
        ell_col=ell_col.astype(np.int32), boundary_face=bids.astype(np.int32), face_dvec=face_dvec,
    )
