"""ORACLE test infrastructure: a stand-in for the pyvista grid members that warp_cfd's
preprocess/mesh.py reads (mesh.py:17-43, :201): ``cells_dict``, ``points``,
``cell_centers().points``, ``compute_cell_sizes()['Volume']`` and
``cell_neighbors(i, connections='faces')``, for grids of linear hexahedra, wedges or
tetrahedra.

* cell centre: VTK's parametric centre of a linear cell, which is the mean of its nodes;
* volume: the sum over the cell's faces of the tetrahedra spanned by the centre and a
  fan triangulation of the face -- exact for convex cells with planar faces (the
  structured and 2D-extruded grids the fixtures use);
* face neighbours: cells sharing all nodes of a face.
"""
from __future__ import annotations

import enum

import numpy as np


class CellType(enum.IntEnum):
    TETRA = 10
    HEXAHEDRON = 12
    WEDGE = 13


_FACES = {
    CellType.HEXAHEDRON: [[0, 3, 2, 1], [4, 5, 6, 7], [0, 1, 5, 4], [1, 2, 6, 5], [2, 3, 7, 6], [3, 0, 4, 7]],
    CellType.WEDGE: [[0, 1, 2], [3, 5, 4], [0, 3, 4, 1], [1, 4, 5, 2], [2, 5, 3, 0]],
    CellType.TETRA: [[0, 2, 1], [0, 1, 3], [1, 2, 3], [2, 0, 3]],
}


class _Points:
    def __init__(self, points):
        self.points = points


class UnstructuredGrid:
    def __init__(self, cells, celltypes, points):
        cells = np.asarray(cells, dtype=np.int64).ravel()
        celltypes = np.asarray(celltypes, dtype=np.int64).ravel()
        self.cells = cells
        self.celltypes = celltypes
        self.points = np.asarray(points, dtype=np.float64).reshape(-1, 3)
        types = np.unique(celltypes)
        if len(types) != 1:
            raise NotImplementedError("the stand-in holds grids of one cell type")
        n = int(cells[0])
        conn = cells.reshape(-1, n + 1)
        self.cells_dict = {int(types[0]): conn[:, 1:].copy()}
        self._type = CellType(int(types[0]))
        self._conn = conn[:, 1:]
        self._nbrs = None

    @property
    def n_cells(self):
        return self._conn.shape[0]

    def cell_centers(self):
        return _Points(self.points[self._conn].mean(axis=1))

    def compute_cell_sizes(self, length=False, area=False, volume=True):
        pts = self.points[self._conn]                       # (C, n, 3)
        c = pts.mean(axis=1)
        vol = np.zeros(self._conn.shape[0])
        for f in _FACES[self._type]:
            a = pts[:, f[0]]
            for j in range(1, len(f) - 1):
                b, d = pts[:, f[j]], pts[:, f[j + 1]]
                vol += np.abs(np.einsum("ij,ij->i", np.cross(b - a, d - a), a - c)) / 6.0
        return {"Volume": vol}

    def cell_neighbors(self, ind, connections="faces"):
        if connections != "faces":
            raise NotImplementedError(connections)
        if self._nbrs is None:
            owners = {}
            for ci, cell in enumerate(self._conn):
                for f in _FACES[self._type]:
                    owners.setdefault(tuple(sorted(int(cell[k]) for k in f)), []).append(ci)
            nb = [set() for _ in range(self._conn.shape[0])]
            for cs in owners.values():
                for a in cs:
                    nb[a].update(x for x in cs if x != a)
            self._nbrs = [sorted(s) for s in nb]
        return list(self._nbrs[ind])


class StructuredGrid(UnstructuredGrid):
    pass


class Plotter:
    def __init__(self, *a, **k):
        raise RuntimeError("no plotting in the stand-in")
