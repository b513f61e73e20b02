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

# local face tables of mesh.py:69-91 (wedge: its two triangles, then its three quads)
HEX_FACES = np.array([[3, 2, 1, 0], [4, 5, 6, 7], [0, 1, 5, 4],
                      [1, 2, 6, 5], [3, 7, 6, 2], [3, 0, 4, 7]], dtype=np.int32)
TET_FACES = np.array([[2, 1, 0], [0, 1, 3], [3, 2, 0], [1, 2, 3]], dtype=np.int32)
WEDGE_SETS = [np.array([[0, 2, 1], [3, 4, 5]], dtype=np.int32),
              np.array([[0, 3, 5, 2], [1, 2, 5, 4], [0, 1, 4, 3]], dtype=np.int32)]
FACE_SETS = {8: [HEX_FACES], 4: [TET_FACES], 6: WEDGE_SETS}   # by nodes per cell


def _fan(nodes, faces):
    """Fan triangulation from local node 0 (mesh.py:161-183): area, unit normal."""
    fc = nodes[faces]
    v0 = fc[:, :, 0, :]
    area = np.zeros(faces.shape[:2])
    vec = np.zeros(faces.shape[:2] + (3,))
    for i in range(1, faces.shape[-1] - 1):
        nv = 0.5 * np.cross(fc[:, :, i, :] - v0, fc[:, :, i + 1, :] - v0)
        area += np.linalg.norm(nv, axis=-1)
        vec += nv
    return area, vec / area[:, :, None]


def reference_mesh_properties(nodes: np.ndarray, cells: np.ndarray):
    """One cell type per mesh (hex, tetra or wedge, told apart by the nodes per cell).
    Returns a dict of the reference's faces_data/cells_data arrays.

    Float arrays are float64 here (the reference keeps float32); comparisons use a
    tolerance.
    """
    nodes = np.asarray(nodes, dtype=np.float64)
    cells = np.asarray(cells, dtype=np.int64)
    C = cells.shape[0]
    centroids = nodes[cells].mean(axis=1)
    sets = FACE_SETS[cells.shape[1]]
    width = max(t.shape[1] for t in sets)
    uf, cf, ar, nr, fcs = [], [], [], [], []
    shift = 0
    for table in sets:                                           # mesh.py:101-150
        faces = cells[:, table]                                  # mesh.py:112
        faces_sorted = np.sort(faces, axis=2).reshape(-1, table.shape[1])   # mesh.py:115-118
        u, inv = np.unique(faces_sorted, axis=0, return_inverse=True)      # mesh.py:121
        a, n = _fan(nodes, faces)
        fcs.append(nodes[u].mean(axis=1))
        if table.shape[1] < width:
            u = np.hstack([u, -np.ones((u.shape[0], width - table.shape[1]), dtype=u.dtype)])
        uf.append(u)
        cf.append(inv.reshape(C, table.shape[0]) + shift)
        ar.append(a)
        nr.append(n)
        shift += u.shape[0]
    unique_faces = np.concatenate(uf, axis=0)
    cell_face_ids = np.concatenate(cf, axis=1)
    area = np.concatenate(ar, axis=1)
    normal = np.concatenate(nr, axis=1)
    face_centroid = np.concatenate(fcs, axis=0)
    to_face = face_centroid[cell_face_ids] - centroids[:, None, :]
    F = cell_face_ids.shape[1]

    # neighbour pairs (i<j) that share a face (mesh.py:186-205)
    K = unique_faces.shape[0]
    occ: list[list[int]] = [[] for _ in range(K)]
    for c in range(C):
        for f in range(F):
            occ[cell_face_ids[c, f]].append(c)
    pairs = sorted({(min(o), max(o)) for o in occ if len(o) == 2})

    adjacent = -np.ones((K, 2), dtype=np.int64)
    cfi = -np.ones((K, 2), dtype=np.int64)
    distance = -np.ones((K, 3))
    is_boundary = np.ones(K, dtype=np.uint8)
    neighbors = -np.ones((C, F), dtype=np.int64)
    face_side = np.zeros((C, F), dtype=np.int64)
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
