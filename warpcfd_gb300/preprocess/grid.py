"""Synthetic mesh generators and wall grouping.

``create_2D_grid`` keeps the signature of warp_cfd/preprocess/grid.py:8 (a rectangle
``dx`` x ``dy`` split into ``nx`` x ``ny`` hexes, extruded one cell thick by ``dz``)
but builds the structured hex grid directly instead of through gmsh.  Node order in
every hex follows VTK (bottom quad counter-clockwise seen from +z, then the top quad),
so the reference's local face table yields outward normals.

``create_3D_grid`` (a box of nx x ny x nz hexes) and the seeded interior-node jitter
are additions for the 3D cavity and the skewed-mesh cases.  ``define_boundary_walls``
follows grid.py:165-194.
"""
from __future__ import annotations

import numpy as np

from .mesh import HEXAHEDRON, Mesh, UnstructuredGrid


def _hex_connectivity(nx, ny, nz):
    """(nx*ny*nz, 8) VTK hex connectivity on an (nx+1)x(ny+1)x(nz+1) node lattice.

    Cell (i,j,k) has id i + nx*(j + ny*k); node (i,j,k) has id i + (nx+1)*(j + (ny+1)*k).
    """
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    i = i.transpose(2, 1, 0).ravel()
    j = j.transpose(2, 1, 0).ravel()
    k = k.transpose(2, 1, 0).ravel()
    sx, sy = nx + 1, (nx + 1) * (ny + 1)
    n0 = i + sx * j + sy * k
    conn = np.stack([n0, n0 + 1, n0 + 1 + sx, n0 + sx,
                     n0 + sy, n0 + 1 + sy, n0 + 1 + sx + sy, n0 + sx + sy], axis=1)
    return conn.astype(np.int64)


def _lattice(origin, nx, ny, nz, lx, ly, lz):
    x = origin[0] + np.linspace(0.0, lx, nx + 1)
    y = origin[1] + np.linspace(0.0, ly, ny + 1)
    z = origin[2] + np.linspace(0.0, lz, nz + 1)
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)


def jitter_interior_nodes(points, nx, ny, nz, h, fraction, seed, planar_z=False):
    """Move every interior lattice node by up to ``fraction`` of the local edge length.

    ``h`` = (hx, hy, hz) edge lengths.  With ``planar_z`` (one-cell-thick meshes) only
    x and y move, and both z layers get the same in-plane offset, so every face stays
    planar.  Boundary nodes stay put so the domain is unchanged.
    """
    rng = np.random.default_rng(seed)
    pts = points.copy()
    I, J, K = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    I = I.transpose(2, 1, 0).ravel()
    J = J.transpose(2, 1, 0).ravel()
    K = K.transpose(2, 1, 0).ravel()
    if planar_z:
        inner = (I > 0) & (I < nx) & (J > 0) & (J < ny)
        off2 = rng.uniform(-1.0, 1.0, size=((nx + 1) * (ny + 1), 2))
        idx2 = I + (nx + 1) * J
        for d in range(2):
            pts[inner, d] += fraction * h[d] * off2[idx2[inner], d]
    else:
        inner = (I > 0) & (I < nx) & (J > 0) & (J < ny) & (K > 0) & (K < nz)
        off = rng.uniform(-1.0, 1.0, size=(pts.shape[0], 3))
        for d in range(3):
            pts[inner, d] += fraction * h[d] * off[inner, d]
    return pts


def create_2D_grid(origin, nx, ny, dx, dy, dz=0.1, *, element_type="hex", unstructured_wedge=False,
                   display_mesh=False, save=None, gmsh_version2=False, jitter=0.0, seed=0) -> UnstructuredGrid:
    """Rectangle ``dx`` x ``dy`` at ``origin`` with ``nx`` x ``ny`` hexes, one cell (``dz``) thick.

    Same call shape as warp_cfd/preprocess/grid.py:8.  Only ``element_type='hex'`` is
    produced (the only cell type that reaches the reference solver).  ``jitter`` > 0
    moves interior nodes by up to that fraction of the local edge length (seeded).
    """
    if element_type != "hex":
        raise NotImplementedError("create_2D_grid builds hex meshes only")
    pts = _lattice(origin, nx, ny, 1, dx, dy, dz)
    if jitter > 0.0:
        pts = jitter_interior_nodes(pts, nx, ny, 1, (dx / nx, dy / ny, dz), jitter, seed, planar_z=True)
    conn = _hex_connectivity(nx, ny, 1)
    cells = np.hstack([np.full((conn.shape[0], 1), 8), conn]).ravel()
    return UnstructuredGrid(cells, np.full(conn.shape[0], HEXAHEDRON), pts)


def create_3D_grid(origin, nx, ny, nz, lx, ly, lz, *, jitter=0.0, seed=0) -> UnstructuredGrid:
    """Box ``lx`` x ``ly`` x ``lz`` of ``nx`` x ``ny`` x ``nz`` hexes (the 3D cavity case)."""
    pts = _lattice(origin, nx, ny, nz, lx, ly, lz)
    if jitter > 0.0:
        pts = jitter_interior_nodes(pts, nx, ny, nz, (lx / nx, ly / ny, lz / nz), jitter, seed)
    conn = _hex_connectivity(nx, ny, nz)
    cells = np.hstack([np.full((conn.shape[0], 1), 8), conn]).ravel()
    return UnstructuredGrid(cells, np.full(conn.shape[0], HEXAHEDRON), pts)


def define_boundary_walls(m: Mesh):
    """Group boundary faces into '+X','-X','+Y','-Y','+Z','-Z' by outward normal.

    Follows warp_cfd/preprocess/grid.py:165-194 (tolerance 1e-3 on n . axis - 1).
    """
    faces = m.face_properties
    cells = m.cell_properties
    boundary_ids = faces.boundary_face_ids
    face_idx = faces.cell_face_index[boundary_ids, 0]
    cell_ids = faces.adjacent_cells[boundary_ids, 0]
    normals = cells.normal[cell_ids, face_idx].astype(np.float64)
    tol = 1e-3
    walls = {}
    for name, axis in (("+X", [1, 0, 0]), ("-X", [-1, 0, 0]), ("+Y", [0, 1, 0]),
                       ("-Y", [0, -1, 0]), ("+Z", [0, 0, 1]), ("-Z", [0, 0, -1])):
        mask = np.abs(normals @ np.array(axis, dtype=np.float64) - 1) < tol
        walls[name] = boundary_ids[mask]
    m.add_groups(walls, "face")
    return walls
