"""ORACLE (test infrastructure only): loop-style restatement of the reference mesh pass.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use
this package, as the checker.  Nothing in ``warpcfd_gb300`` imports it.

Restates warp_cfd/preprocess/mesh.py:64-302 in the reference's own style
(``np.unique(axis=0)`` on sorted face-node rows, then a Python loop over the sorted
neighbour pairs with ``np.intersect1d``, mesh.py:263-281), so the vectorised
preprocessing in ``warpcfd_gb300.preprocess.mesh`` can be checked against it on small
meshes.  Neighbour pairs come from shared faces, which is what pyvista's
``cell_neighbors(i, 'faces')`` returns for a conforming mesh.
"""
from __future__ import annotations

import numpy as np

HEX_FACES = np.array([[3, 2, 1, 0], [4, 5, 6, 7], [0, 1, 5, 4],
                      [1, 2, 6, 5], [3, 7, 6, 2], [3, 0, 4, 7]], dtype=np.int32)


def reference_mesh_properties(nodes: np.ndarray, cells: np.ndarray):
    """Hex meshes only.  Returns a dict of the reference's faces_data/cells_data arrays.

    Float arrays are float64 here (the reference keeps float32); comparisons use a
    tolerance.
    """
    nodes = np.asarray(nodes, dtype=np.float64)
    cells = np.asarray(cells, dtype=np.int64)
    C = cells.shape[0]
    centroids = nodes[cells].mean(axis=1)
    faces = cells[:, HEX_FACES]                                  # mesh.py:112
    faces_sorted = np.sort(faces, axis=2).reshape(-1, 4)         # mesh.py:115-118
    unique_faces, inv = np.unique(faces_sorted, axis=0, return_inverse=True)  # mesh.py:121
    cell_face_ids = inv.reshape(C, 6)
    # fan triangulation (mesh.py:161-183)
    fc = nodes[faces]
    v0 = fc[:, :, 0, :]
    areas, vecs = [], []
    for i in range(1, 3):
        nv = 0.5 * np.cross(fc[:, :, i, :] - v0, fc[:, :, i + 1, :] - v0)
        areas.append(np.linalg.norm(nv, axis=-1))
        vecs.append(nv)
    area = sum(areas)
    normal = sum(vecs) / area[:, :, None]
    face_centroid = nodes[unique_faces].mean(axis=1)
    to_face = face_centroid[cell_face_ids] - centroids[:, None, :]

    # neighbour pairs (i<j) that share a face (mesh.py:186-205)
    K = unique_faces.shape[0]
    occ: list[list[int]] = [[] for _ in range(K)]
    for c in range(C):
        for f in range(6):
            occ[cell_face_ids[c, f]].append(c)
    pairs = sorted({(min(o), max(o)) for o in occ if len(o) == 2})

    adjacent = -np.ones((K, 2), dtype=np.int64)
    cfi = -np.ones((K, 2), dtype=np.int64)
    distance = -np.ones((K, 3))
    is_boundary = np.ones(K, dtype=np.uint8)
    neighbors = -np.ones((C, 6), dtype=np.int64)
    face_side = np.zeros((C, 6), dtype=np.int64)
    nnz = np.ones(C, dtype=np.int64)
    for i, j in pairs:                                           # mesh.py:263-281
        fid, ii, jj = np.intersect1d(cell_face_ids[i], cell_face_ids[j], return_indices=True)
        assert ii.shape[0] == 1
        neighbors[i, ii[0]] = j
        neighbors[j, jj[0]] = i
        face_side[i, ii[0]] = 0
        face_side[j, jj[0]] = 1
        nnz[i] += 1
        nnz[j] += 1
        distance[fid] = centroids[j] - centroids[i]
        is_boundary[fid] = 0
        adjacent[fid] = [i, j]
        cfi[fid] = [ii[0], jj[0]]
    for c, f in np.argwhere(neighbors == -1):                    # mesh.py:285-288
        fid = cell_face_ids[c, f]
        adjacent[fid, 0] = c
        cfi[fid, 0] = f
    ids = np.arange(K)
    m = neighbors != -1
    return dict(
        unique_faces=unique_faces, cell_faces=cell_face_ids, normal=normal, area=area,
        face_centroid=face_centroid, to_face=to_face, centroids=centroids,
        adjacent=adjacent, cell_face_index=cfi, distance=distance, is_boundary=is_boundary,
        neighbors=neighbors, face_side=face_side, nnz_per_cell=nnz,
        face_offset_index=np.cumsum(m, axis=1) * m,
        boundary_face_ids=ids[is_boundary == 1], internal_face_ids=ids[is_boundary == 0],
    )
