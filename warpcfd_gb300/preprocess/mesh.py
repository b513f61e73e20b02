"""Unstructured-mesh preprocessing: cells -> unique faces, owner/neighbour, geometry.

Host-side numpy, run once per mesh. It produces every topology and geometry array
the finite-volume step consumes, with the same meaning and the same numbering as
``warp_cfd.preprocess.Mesh`` (warp_cfd/preprocess/mesh.py:17-302):

* unique faces are numbered in the lexicographic order of their sorted node ids
  (``np.unique(axis=0)`` at mesh.py:121);
* per (cell, local face slot) the fan-triangulated area and outward normal are taken
  from the cell-local node order (mesh.py:161-183), so normals point out of the cell;
* owner = lower cell id, neighbour = higher (pairs sorted at mesh.py:205);
* ``nnz_per_cell`` = 1 + number of internal faces; ``face_offset_index`` numbers the
  internal slots of a cell 1, 2, ... in slot order and is 0 on boundary slots
  (mesh.py:299-300).

Unlike the reference it needs neither pyvista nor gmsh, and the owner/neighbour pass
is vectorised (the reference walks the neighbour pairs in a Python loop,
mesh.py:263-281), so a 2.1M-cell hex mesh preprocesses in seconds.

Mixed meshes (hexahedra, wedges and tetrahedra in one grid; the reference accepts one
cell type, mesh.py:20) are an extension.  Cells keep the grid's order; every cell has
F = the largest face count of the types present slots, its own faces first in its
type's table order and then null slots (face id -1, zero area and normal, neighbour -1,
``slot_valid`` False).  Faces are numbered triangles first, then quadrilaterals, each
set in lexicographic order of its sorted node ids -- for a single-type mesh exactly the
reference's numbering (a wedge mesh's triangle set precedes its quad set there too).
"""
from __future__ import annotations

import numpy as np

# VTK cell type ids (the same integers pyvista.CellType uses).
TETRA = 10
HEXAHEDRON = 12
WEDGE = 13

CELL_TYPE_NAMES = {TETRA: "TETRA", HEXAHEDRON: "HEXAHEDRON", WEDGE: "WEDGE"}

# Local face -> local node tables.  They must equal the reference's tables
# (warp_cfd/preprocess/mesh.py:69-91) because the local slot order fixes the
# per-cell face order, the CSR column order and every outward normal.
HEX_FACES = np.array([[3, 2, 1, 0],
                      [4, 5, 6, 7],
                      [0, 1, 5, 4],
                      [1, 2, 6, 5],
                      [3, 7, 6, 2],
                      [3, 0, 4, 7]], dtype=np.int32)
TET_FACES = np.array([[2, 1, 0],
                      [0, 1, 3],
                      [3, 2, 0],
                      [1, 2, 3]], dtype=np.int32)
# wedge: two triangles then three quads
WEDGE_TRI_FACES = np.array([[0, 2, 1], [3, 4, 5]], dtype=np.int32)
WEDGE_QUAD_FACES = np.array([[0, 3, 5, 2], [1, 2, 5, 4], [0, 1, 4, 3]], dtype=np.int32)

NODES_PER_CELL = {TETRA: 4, HEXAHEDRON: 8, WEDGE: 6}

# per cell type: its local faces in slot order
CELL_FACES = {HEXAHEDRON: [tuple(f) for f in HEX_FACES],
              TETRA: [tuple(f) for f in TET_FACES],
              WEDGE: [tuple(f) for f in WEDGE_TRI_FACES] + [tuple(f) for f in WEDGE_QUAD_FACES]}


def padded_connectivity(grid):
    """(C, 8) int64 node ids in the grid's cell order, -1 past each cell's node count,
    and the (C,) VTK type of every cell.  Reads ``celltypes`` and the flat VTK ``cells``
    array ([n, i0 .. i(n-1), n, ...]) of a pyvista-style grid."""
    types = np.asarray(grid.celltypes, dtype=np.int64).ravel()
    flat = np.asarray(grid.cells, dtype=np.int64).ravel()
    C = types.shape[0]
    npc = np.zeros(C, dtype=np.int64)
    for t, n in NODES_PER_CELL.items():
        npc[types == t] = n
    if np.any(npc == 0):
        raise AssertionError("only Tetra and Hexahedron and Wedge elements are supported")
    start = np.concatenate([[0], np.cumsum(npc + 1)[:-1]]) + 1
    if flat.shape[0] != int((npc + 1).sum()) or np.any(flat[start - 1] != npc):
        raise ValueError("inconsistent node counts in cell connectivity")
    conn = -np.ones((C, 8), dtype=np.int64)
    for j in range(8):
        has = npc > j
        conn[has, j] = flat[start[has] + j]
    return conn, types


class UnstructuredGrid:
    """Minimal stand-in for ``pyvista.UnstructuredGrid`` (cells, celltypes, points).

    ``cells`` is VTK's flat connectivity ``[n, i0, ..., i(n-1), n, ...]``, exactly what
    ``create_2D_grid`` hands to pyvista at warp_cfd/preprocess/grid.py:156-159.
    Only the members the mesh preprocessing reads are provided.
    """

    def __init__(self, cells, celltypes, points):
        cells = np.asarray(cells, dtype=np.int64).ravel()
        celltypes = np.asarray(celltypes, dtype=np.int64).ravel()
        self.cells = cells
        self.points = np.asarray(points, dtype=np.float64).reshape(-1, 3)
        self.celltypes = celltypes
        types = np.unique(celltypes)
        self.cells_dict = {}
        if len(types) == 1:
            npc = int(cells[0])
            conn = cells.reshape(-1, npc + 1)
            if not np.all(conn[:, 0] == npc):
                raise ValueError("inconsistent node counts in cell connectivity")
            self.cells_dict[int(types[0])] = conn[:, 1:].astype(np.int64)
        else:
            pos = 0
            per_type: dict[int, list] = {int(t): [] for t in types}
            for t in celltypes:
                n = int(cells[pos])
                per_type[int(t)].append(cells[pos + 1: pos + 1 + n])
                pos += n + 1
            self.cells_dict = {t: np.array(v, dtype=np.int64) for t, v in per_type.items()}

    @property
    def n_cells(self):
        return int(sum(v.shape[0] for v in self.cells_dict.values()))

    @property
    def n_points(self):
        return int(self.points.shape[0])


class group:
    """Named set of ids (warp_cfd/preprocess/mesh.py:8-15)."""

    def __init__(self, name, ids, type) -> None:
        self.name = name
        self.ids = ids
        self.type = type


class cells_data:
    """Per-cell arrays; member names and meanings follow mesh.py:306-366.

    faces (C,F) unique-face id per local slot; normal (C,F,3); area (C,F);
    neighbors (C,F) (-1 = boundary); centroids (C,3); volumes (C,);
    nodes (C,N); cell_centroid_to_face_centroid (C,F,3); face_side (C,F) 0 = owner;
    nnz_per_cell (C,); face_offset_index (C,F).
    """


class faces_data:
    """Per-face arrays; member names and meanings follow mesh.py:408-469.

    unique_faces (K,N); centroid (K,3); is_boundary (K,) uint8;
    boundary_face_ids (B,); internal_face_ids (K-B,); adjacent_cells (K,2);
    cell_face_index (K,2); num_nodes (K,); distance (K,3) owner->neighbour
    centroid vector (-1 on boundary faces).
    """


def _face_normal_and_area(face_nodes: np.ndarray, nodes: np.ndarray):
    """Fan triangulation from local node 0, as mesh.py:161-183.

    area = sum of triangle areas; normal = (sum of triangle vector areas) / area.
    Computed in float64 and returned as float64.
    """
    coords = nodes[face_nodes]  # (..., n, 3)
    v0 = coords[..., 0, :]
    area = np.zeros(face_nodes.shape[:-1], dtype=np.float64)
    vec = np.zeros(face_nodes.shape[:-1] + (3,), dtype=np.float64)
    for i in range(1, face_nodes.shape[-1] - 1):
        nv = 0.5 * np.cross(coords[..., i, :] - v0, coords[..., i + 1, :] - v0)
        area += np.linalg.norm(nv, axis=-1)
        vec += nv
    normal = vec / area[..., None]
    return area, normal


def _unique_rows(sorted_rows: np.ndarray):
    """Unique rows in lexicographic order plus the inverse map.

    Equivalent to ``np.unique(rows, axis=0, return_inverse=True)`` for non-negative
    int rows (the ordering mesh.py:121 produces), but via a packed-key lexsort so a
    12.6M x 4 face table sorts in a couple of seconds.
    """
    n, m = sorted_rows.shape
    r = sorted_rows.astype(np.int64)
    keys = []
    # pack two 32-bit ids per 64-bit key, most significant column first
    for j in range(0, m, 2):
        if j + 1 < m:
            keys.append((r[:, j] << 32) | r[:, j + 1])
        else:
            keys.append(r[:, j] << 32)
    order = np.lexsort(tuple(reversed(keys)))
    ks = [k[order] for k in keys]
    new = np.ones(n, dtype=bool)
    if n > 1:
        same = np.ones(n - 1, dtype=bool)
        for k in ks:
            same &= k[1:] == k[:-1]
        new[1:] = ~same
    group_id = np.cumsum(new) - 1
    inverse = np.empty(n, dtype=np.int64)
    inverse[order] = group_id
    unique = sorted_rows[order[new]]
    return unique, inverse


class Mesh:
    """Mesh preprocessing with the API of ``warp_cfd.preprocess.Mesh`` (mesh.py:17-302).

    ``grid`` is anything with ``.points`` (N,3) and ``.cells_dict`` {vtk type: (C,n)}:
    a pyvista grid, or :class:`UnstructuredGrid`.  A grid of one cell type is handled as
    the reference handles it (mesh.py:17-43); a grid that mixes types also needs the
    flat ``cells`` and ``celltypes`` arrays, and then ``cells`` is (C, 8) padded with -1,
    ``cell_types`` the VTK type per cell and ``cellType`` ('MIXED', 0).  ``device`` (a
    CUDA device) runs the face matching and the geometry on the GPU (libwcfd's mesh pass,
    for meshes of millions of cells) with bit-identical topology.
    """

    def __init__(self, grid, dtype=np.float32, device=None) -> None:
        cells_dict = grid.cells_dict
        self.device = device
        self.float_dtype = np.float32
        self.int_dtype = np.int32
        self.dtype = dtype
        self.pyvista_mesh = grid
        points = np.asarray(grid.points, dtype=np.float64)
        self._nodes64 = points
        self.nodes = points.astype(self.float_dtype)
        types = [int(t) for t in cells_dict.keys()]
        if any(t not in (HEXAHEDRON, TETRA, WEDGE) for t in types):
            raise AssertionError("only Tetra and Hexahedron and Wedge elements are supported")
        if len(types) == 1:
            celltype = types[0]
            self.cellType = (CELL_TYPE_NAMES[celltype], celltype)
            self.cells = np.asarray(cells_dict[celltype], dtype=self.int_dtype)
            self.cell_types = np.full(self.cells.shape[0], celltype, dtype=np.int32)
        else:
            if not (hasattr(grid, "cells") and hasattr(grid, "celltypes")):
                raise AssertionError("a mixed-type grid needs its flat cells and celltypes arrays")
            conn, ctypes = padded_connectivity(grid)
            self.cellType = ("MIXED", 0)
            self.cells = conn.astype(self.int_dtype)
            self.cell_types = ctypes.astype(np.int32)
        if device is None:
            self._centroids64 = self._host_centroids()
            self.cell_centroids = self._centroids64.astype(self.float_dtype)
        self.groups: dict[str, group] = {}
        self.gridType = "Unstructured"
        self.face_properties, self.cell_properties = self.get_mesh_properties()
        self.cell_volumes = self.cell_properties.volumes

    def _host_centroids(self):
        """VTK's cell centre of a linear cell: its parametric centre = the node mean."""
        points = self._nodes64
        if self.cellType[1] != 0:
            return points[self.cells.astype(np.int64)].mean(axis=1)
        conn = self.cells.astype(np.int64)
        real = conn >= 0
        pts = points[np.maximum(conn, 0)] * real[..., None]
        return pts.sum(axis=1) / real.sum(axis=1)[:, None]

    @classmethod
    def from_arrays(cls, nodes, cells, cell_type=HEXAHEDRON):
        cells = np.asarray(cells)
        flat = np.hstack([np.full((cells.shape[0], 1), cells.shape[1]), cells]).ravel()
        return cls(UnstructuredGrid(flat, np.full(cells.shape[0], cell_type), nodes))

    @property
    def dimension(self):
        assert self.nodes.shape[-1] == 3, "Only 3 Dimensional Meshes are supported"
        return 3

    @property
    def num_cells(self):
        return int(self.cells.shape[0])

    @property
    def num_faces(self):
        return int(self.face_properties.unique_faces.shape[0])

    def add_group(self, name, id, group_type):
        group_types = {"face", "cell", "point", "edge"}
        assert group_type in group_types, "group_type must be one of the following: {face,cell,point,edge}"
        assert name not in self.groups.keys(), "name for group already exists!"
        self.groups[name] = group(name, np.asarray(id), group_type)

    def add_groups(self, dic: dict, group_type):
        for name, id in dic.items():
            self.add_group(name, id, group_type)

    # ------------------------------------------------------------------ faces
    def _face_groups(self, npf):
        """[(cell ids, slots, (Ct, Fs, npf) local node ids)] of every cell type's faces
        with ``npf`` nodes, in the type order of the first appearance in the grid."""
        groups = []
        types = self.cell_types
        uniq, first = np.unique(types, return_index=True)
        for t in uniq[np.argsort(first)]:
            faces = CELL_FACES[int(t)]
            slots = [j for j, f in enumerate(faces) if len(f) == npf]
            if not slots:
                continue
            ids = np.nonzero(types == t)[0] if len(uniq) > 1 else np.arange(types.shape[0])
            table = np.array([faces[j] for j in slots], dtype=np.int64)
            groups.append((ids, np.array(slots, dtype=np.int64), table))
        return groups

    @property
    def faces_per_cell(self):
        return max(len(CELL_FACES[int(t)]) for t in np.unique(self.cell_types))

    def get_faces(self):
        """Unique faces and per-(cell,slot) face ids, areas, normals (mesh.py:64-159).

        Triangles are numbered before quadrilaterals; null slots (cells with fewer faces
        than F) get face id -1 and zero geometry."""
        cells = self.cells.astype(np.int64)
        C = cells.shape[0]
        F = self.faces_per_cell
        sets = [(npf, self._face_groups(npf)) for npf in (3, 4)]
        sets = [(npf, g) for npf, g in sets if g]
        N = max(npf for npf, _ in sets)
        cell_face_ids = -np.ones((C, F), dtype=np.int64)
        area = np.zeros((C, F), dtype=np.float64)
        normal = np.zeros((C, F, 3), dtype=np.float64)
        to_face = np.zeros((C, F, 3), dtype=np.float64)
        shift = 0
        parts = []
        single = len(np.unique(self.cell_types)) == 1
        for npf, groups in sets:
            rows, row_cell, row_slot = [], [], []
            for ids, slots, table in groups:
                # a type's faces of one node count occupy consecutive slots
                sl = slice(int(slots[0]), int(slots[-1]) + 1)
                faces = cells[ids][:, table] if not single else cells[:, table]  # (Ct,Fs,npf)
                a, n = _face_normal_and_area(faces, self._nodes64)
                if single:
                    area[:, sl], normal[:, sl] = a, n
                else:
                    area[ids, sl], normal[ids, sl] = a, n
                rows.append(faces.reshape(-1, npf))
                row_cell.append(np.repeat(ids, len(slots)))
                row_slot.append(np.tile(slots, len(ids)))
            faces = rows[0] if len(rows) == 1 else np.concatenate(rows, axis=0)
            fsorted = np.sort(faces, axis=1)
            unique, inv = _unique_rows(fsorted)
            fcent = self._nodes64[unique].mean(axis=1)
            if single:
                sl = slice(int(groups[0][1][0]), int(groups[0][1][-1]) + 1)
                ids2 = inv.reshape(C, -1)
                cell_face_ids[:, sl] = ids2 + shift
                to_face[:, sl] = fcent[ids2] - self._centroids64[:, None, :]
            else:
                rc, rs = np.concatenate(row_cell), np.concatenate(row_slot)
                cell_face_ids[rc, rs] = inv + shift
                to_face[rc, rs] = fcent[inv] - self._centroids64[rc]
            if N - npf > 0:
                unique = np.hstack([unique, -np.ones((unique.shape[0], N - npf), dtype=unique.dtype)])
            parts.append((unique, np.full(len(unique), npf, dtype=np.int32), fcent))
            shift += len(unique)
        cat0 = lambda i: np.concatenate([p[i] for p in parts], axis=0)
        return (cat0(0).astype(np.int32), cell_face_ids.astype(np.int32), area, normal,
                cat0(1), cat0(2), to_face)

    def get_mesh_properties(self):
        """faces_data, cells_data (mesh.py:186-302); face matching and geometry on the host,
        or on ``device`` (a CUDA device) through libwcfd's mesh pass."""
        if self.device is not None:
            from .device_pass import device_topology
            raw = device_topology(self, self.device)
            self._centroids64 = raw["centroid"]
            self.cell_centroids = self._centroids64.astype(self.float_dtype)
        else:
            raw = self._host_topology()
        return self._assemble(raw)

    def _host_topology(self):
        unique_faces, cell_face_ids, area, normal, nodes_per_face, face_centroid, to_face = self.get_faces()
        C, F = cell_face_ids.shape
        K = unique_faces.shape[0]

        # every unique face occurs once (boundary) or twice (internal) in the (C,F)
        # table; a stable sort of the flat table puts the lower cell id first
        flat = cell_face_ids.ravel().astype(np.int64)
        valid = flat >= 0
        if valid.all():
            order = np.argsort(flat, kind="stable")
        else:
            vidx = np.nonzero(valid)[0]
            order = vidx[np.argsort(flat[vidx], kind="stable")]
        sf = flat[order]
        counts = np.bincount(sf, minlength=K)
        if np.any(counts > 2) or np.any(counts == 0):
            raise AssertionError("a face is shared by more than two cells or is orphaned")
        first = np.searchsorted(sf, np.arange(K), side="left")
        first_pos = order[first]  # flat index of first occurrence
        second_pos = np.where(counts == 2, order[np.minimum(first + 1, len(order) - 1)], -1)
        own_cell = first_pos // F
        own_slot = first_pos % F
        internal = counts == 2
        nb_cell = np.where(internal, second_pos // F, -1)
        nb_slot = np.where(internal, second_pos % F, -1)
        if np.any(internal & (nb_cell == own_cell)):
            raise AssertionError("a cell shares a face with itself")
        return dict(unique_faces=unique_faces, cell_face_ids=cell_face_ids, area=area, normal=normal,
                    nodes_per_face=nodes_per_face, face_centroid=face_centroid, to_face=to_face,
                    own_cell=own_cell, own_slot=own_slot, nb_cell=nb_cell, nb_slot=nb_slot, volume=None)

    def _assemble(self, raw):
        unique_faces, cell_face_ids = raw["unique_faces"], raw["cell_face_ids"]
        area, normal, to_face = raw["area"], raw["normal"], raw["to_face"]
        nodes_per_face, face_centroid = raw["nodes_per_face"], raw["face_centroid"]
        own_cell, own_slot, nb_cell, nb_slot = raw["own_cell"], raw["own_slot"], raw["nb_cell"], raw["nb_slot"]
        C, F = cell_face_ids.shape
        K = unique_faces.shape[0]
        fi = self.int_dtype
        ff = self.float_dtype
        internal = nb_cell >= 0

        faces = faces_data()
        cells = cells_data()
        cells.num_cells = C
        cells.faces_per_cell = F
        cells.nodes_per_face = unique_faces.shape[-1]
        cells.dimension = 3
        faces.num_faces = K
        faces.dimension = 3
        faces.nodes_per_face = unique_faces.shape[-1]
        faces.unique_faces = unique_faces
        faces.centroid = face_centroid.astype(ff)
        faces.num_nodes = nodes_per_face.astype(fi)
        faces.is_boundary = (~internal).astype(np.uint8)
        faces.adjacent_cells = np.stack([own_cell, nb_cell], axis=1).astype(fi)
        faces.cell_face_index = np.stack([own_slot, nb_slot], axis=1).astype(fi)
        # owner -> neighbour centroid vector, the difference of the float32 centroids
        # taken in float32 as the reference takes it (mesh.py:276)
        dist = np.full((K, 3), -1.0, dtype=ff)
        ii = np.nonzero(internal)[0]
        c32 = self._centroids64.astype(ff)
        dist[ii] = c32[nb_cell[ii]] - c32[own_cell[ii]]
        faces.distance = dist
        face_ids = np.arange(K, dtype=fi)
        faces.boundary_face_ids = face_ids[~internal]
        faces.internal_face_ids = face_ids[internal]
        faces.num_boundary_faces = int(len(faces.boundary_face_ids))

        neighbors = -np.ones((C, F), dtype=np.int64)
        face_side = np.zeros((C, F), dtype=np.int64)
        neighbors[own_cell[ii], own_slot[ii]] = nb_cell[ii]
        neighbors[nb_cell[ii], nb_slot[ii]] = own_cell[ii]
        face_side[nb_cell[ii], nb_slot[ii]] = 1
        cells.centroids = self.cell_centroids
        cells.nodes = self.cells
        cells.faces = cell_face_ids.astype(fi)
        cells.normal = normal.astype(ff)
        cells.area = area.astype(ff)
        cells.cell_centroid_to_face_centroid = to_face.astype(ff)
        cells.neighbors = neighbors.astype(fi)
        cells.face_side = face_side.astype(fi)
        cells.slot_valid = (cell_face_ids >= 0)
        cells.cell_types = self.cell_types
        cells.nnz_per_cell = (1 + (neighbors != -1).sum(axis=1)).astype(fi)
        m = neighbors != -1
        cells.face_offset_index = (np.cumsum(m, axis=1) * m).astype(fi)
        # volume by the divergence theorem over the fan-triangulated faces
        # (equal to VTK's cell size for cells with planar faces)
        if raw["volume"] is None:
            fc_vec = (normal * area[..., None])  # outward vector area per slot
            vol = np.abs(np.einsum("cfk,cfk->c", fc_vec, face_centroid[np.maximum(cell_face_ids, 0)]) / 3.0)
        else:
            vol = raw["volume"]
        cells.volumes = vol.astype(ff)
        self._geometry64 = dict(area=area, normal=normal, to_face=to_face, face_centroid=face_centroid,
                                volume=vol, centroid=self._centroids64)
        return faces, cells
