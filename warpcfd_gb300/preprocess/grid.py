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

from .mesh import HEXAHEDRON, TETRA, WEDGE, Mesh, UnstructuredGrid


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


def _cells_with_prisms(conn, split):
    """VTK cells of a hex lattice in which the hexes where ``split`` is True are cut into
    two wedges along the diagonal (node 0 -> node 2) of their bottom quad.  A wedge keeps
    VTK's order (triangle 0-1-2 counter-clockwise seen from its opposite triangle 3-4-5),
    so the wedge face table yields outward normals.  Cells stay in lattice order, the two
    wedges of a hex one after the other."""
    C = conn.shape[0]
    split = np.asarray(split, dtype=bool)
    n_out = C + int(split.sum())
    first = np.arange(C) + np.concatenate([[0], np.cumsum(split)[:-1]])  # output id of each hex's first cell
    types = np.full(n_out, HEXAHEDRON, dtype=np.int64)
    types[first[split]] = WEDGE
    types[first[split] + 1] = WEDGE
    npc = np.where(types == HEXAHEDRON, 8, 6)
    flat = np.empty(int((npc + 1).sum()), dtype=np.int64)
    start = np.concatenate([[0], np.cumsum(npc + 1)[:-1]])
    flat[start] = npc
    h = ~split
    for j in range(8):
        flat[start[first[h]] + 1 + j] = conn[h, j]
    a = conn[split][:, [0, 1, 2, 4, 5, 6]]
    b = conn[split][:, [0, 2, 3, 4, 6, 7]]
    for j in range(6):
        flat[start[first[split]] + 1 + j] = a[:, j]
        flat[start[first[split] + 1] + 1 + j] = b[:, j]
    return flat, types


# Kuhn subdivision of a hex into six tetrahedra around its 0-6 diagonal (VTK hex order);
# the same diagonal direction in every cell of a lattice gives a conforming mesh
_KUHN = np.array([[0, 1, 2, 6], [0, 2, 3, 6], [0, 3, 7, 6], [0, 7, 4, 6], [0, 4, 5, 6], [0, 5, 1, 6]])


def _tets_of_hexes(conn, pts):
    """(6C, 4) tetrahedra of a hex lattice, each ordered as VTK orders a tetra (nodes 0-1-2
    counter-clockwise seen from node 3: positive signed volume), so the tetra face table
    yields outward normals."""
    tets = conn[:, _KUHN].reshape(-1, 4)
    p = pts[tets]
    vol = np.einsum("ij,ij->i", np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]), p[:, 3] - p[:, 0])
    neg = vol < 0
    tets[neg, 1], tets[neg, 2] = tets[neg, 2].copy(), tets[neg, 1].copy()
    return tets


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

    Same call shape as warp_cfd/preprocess/grid.py:8.  ``element_type`` 'hex' (the only
    cell type the reference's examples run), 'wedge' (every quad cut into two
    triangles, extruded: a prism mesh) or 'mixed' (the quads of the right half cut, a
    hex/prism mesh).  ``jitter`` > 0 moves interior nodes by up to that fraction of the
    local edge length (seeded).
    """
    if element_type not in ("hex", "wedge", "mixed"):
        raise NotImplementedError("create_2D_grid builds hex, wedge and mixed hex/wedge meshes")
    pts = _lattice(origin, nx, ny, 1, dx, dy, dz)
    if jitter > 0.0:
        pts = jitter_interior_nodes(pts, nx, ny, 1, (dx / nx, dy / ny, dz), jitter, seed, planar_z=True)
    conn = _hex_connectivity(nx, ny, 1)
    if element_type == "hex":
        cells = np.hstack([np.full((conn.shape[0], 1), 8), conn]).ravel()
        return UnstructuredGrid(cells, np.full(conn.shape[0], HEXAHEDRON), pts)
    i = np.arange(conn.shape[0]) % nx
    split = np.ones(conn.shape[0], dtype=bool) if element_type == "wedge" else i >= nx // 2
    cells, types = _cells_with_prisms(conn, split)
    return UnstructuredGrid(cells, types, pts)


def create_3D_grid(origin, nx, ny, nz, lx, ly, lz, *, jitter=0.0, seed=0,
                   prism_fraction=0.0, element_type="hex") -> UnstructuredGrid:
    """Box ``lx`` x ``ly`` x ``lz`` of ``nx`` x ``ny`` x ``nz`` hexes (the 3D cavity case).

    ``prism_fraction`` > 0 cuts that fraction of the hexes (a seeded random choice) into
    two wedges each: a mixed hex/prism mesh.  With ``jitter`` the cut hexes' faces are no
    longer planar, so jitter and prisms are not combined.  ``element_type='tetra'`` cuts
    every hex into six tetrahedra (Kuhn subdivision; faces are triangles, so jitter is
    allowed)."""
    if prism_fraction > 0.0 and jitter > 0.0:
        raise ValueError("prism_fraction needs planar hex faces: use jitter = 0")
    if element_type not in ("hex", "tetra"):
        raise NotImplementedError("create_3D_grid builds hex, mixed hex/prism and tetra meshes")
    pts = _lattice(origin, nx, ny, nz, lx, ly, lz)
    if jitter > 0.0:
        pts = jitter_interior_nodes(pts, nx, ny, nz, (lx / nx, ly / ny, lz / nz), jitter, seed)
    conn = _hex_connectivity(nx, ny, nz)
    if element_type == "tetra":
        tets = _tets_of_hexes(conn, pts)
        cells = np.hstack([np.full((tets.shape[0], 1), 4), tets]).ravel()
        return UnstructuredGrid(cells, np.full(tets.shape[0], TETRA), pts)
    if prism_fraction > 0.0:
        split = np.random.default_rng(seed).random(conn.shape[0]) < prism_fraction
        cells, types = _cells_with_prisms(conn, split)
        return UnstructuredGrid(cells, types, pts)
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


def _merge_nodes(points2d, tol=1e-9):
    """Unique 2D points (rounded to ``tol``) and the map from input to unique index."""
    key = np.round(points2d / tol).astype(np.int64)
    uniq, inv = np.unique(key, axis=0, return_inverse=True)
    pts = np.zeros((len(uniq), 2))
    np.add.at(pts, inv.ravel(), points2d)
    cnt = np.bincount(inv.ravel(), minlength=len(uniq))
    return pts / cnt[:, None], inv.ravel()


def _block(xy):
    """Quads of a structured (ni+1, nj+1, 2) node block, counter-clockwise."""
    ni, nj = xy.shape[0] - 1, xy.shape[1] - 1
    idx = np.arange((ni + 1) * (nj + 1)).reshape(ni + 1, nj + 1)
    q = np.stack([idx[:-1, :-1], idx[1:, :-1], idx[1:, 1:], idx[:-1, 1:]], axis=-1).reshape(-1, 4)
    return xy.reshape(-1, 2), q


def create_cylinder_channel_grid(scale=1.0, dz=0.01, jitter=0.1, seed=0, length=2.2, height=0.41,
                                 center=(0.2, 0.2), diameter=0.1, box=0.1, prisms=False):
    """2D-extruded channel ``length`` x ``height`` around a cylinder (one cell thick).

    Nine structured blocks: an O-grid of four quadrants between the cylinder (radius
    diameter/2) and a square of half-width ``box`` around it, and eight rectangular blocks
    filling the rest of the channel, all with matching nodes.  All hex by default:
    ``scale`` = 1.0 gives about 96k cells, 1.625 about 254k.  With ``prisms`` every quad
    of the eight rectangular blocks is cut into two triangles, so the far field is prisms
    (wedges) and the O-grid hexes: a prism/hex mesh (``scale`` = 1.15 gives about 245k
    cells).  Interior nodes (not on the walls, inlet, outlet or the cylinder) move by up to
    ``jitter`` of their shortest incident edge, from ``seed``.

    Returns (grid, info) with info['cylinder'] = (cx, cy, r) for grouping the cylinder faces.
    """
    cx, cy = center
    r0 = diameter / 2.0
    x0, x1, y0, y1 = cx - box, cx + box, cy - box, cy + box
    h = 2 * box / max(8, int(round(64 * scale)))
    nB = int(round(2 * box / h))
    nA = max(2, int(round(x0 / h)))
    nC = max(2, int(round((length - x1) / h)))
    na = max(2, int(round(y0 / h)))
    nc = max(2, int(round((height - y1) / h)))
    nr = max(4, int(round(32 * scale)))
    xs = [np.linspace(0.0, x0, nA + 1), np.linspace(x0, x1, nB + 1), np.linspace(x1, length, nC + 1)]
    ys = [np.linspace(0.0, y0, na + 1), np.linspace(y0, y1, nB + 1), np.linspace(y1, height, nc + 1)]
    pts_list, quads_list, far_list, off = [], [], [], 0
    for bi in range(3):
        for bj in range(3):
            if bi == 1 and bj == 1:
                continue
            X, Y = np.meshgrid(xs[bi], ys[bj], indexing="ij")
            p, q = _block(np.stack([X, Y], axis=-1))
            pts_list.append(p)
            quads_list.append(q + off)
            far_list.append(np.ones(len(q), dtype=bool))
            off += len(p)
    # O-grid: quadrant k spans angles [th0, th0 + 90deg]; the outer edge is a box side
    t = np.linspace(0.0, 1.0, nB + 1)
    s = np.linspace(0.0, 1.0, nr + 1)
    s = s ** 1.5                                      # cluster radial cells at the cylinder
    sides = [  # (angle start, outer edge start point, outer edge end point)
        (-np.pi / 4, (x1, y0), (x1, y1)),
        (np.pi / 4, (x1, y1), (x0, y1)),
        (3 * np.pi / 4, (x0, y1), (x0, y0)),
        (5 * np.pi / 4, (x0, y0), (x1, y0)),
    ]
    for th0, pa, pb in sides:
        th = th0 + t * (np.pi / 2)
        inner = np.stack([cx + r0 * np.cos(th), cy + r0 * np.sin(th)], axis=-1)        # (nB+1, 2)
        outer = np.stack([pa[0] + t * (pb[0] - pa[0]), pa[1] + t * (pb[1] - pa[1])], axis=-1)
        blk = inner[:, None, :] + s[None, :, None] * (outer - inner)[:, None, :]       # (nB+1, nr+1, 2)
        # index order (i along the arc, j outward) is clockwise for this orientation:
        # flip j so quads come out counter-clockwise
        p, q = _block(blk[:, ::-1, :])
        pts_list.append(p)
        quads_list.append(q + off)
        far_list.append(np.zeros(len(q), dtype=bool))
        off += len(p)
    pts2, inv = _merge_nodes(np.concatenate(pts_list))
    quads = inv[np.concatenate(quads_list)]
    # counter-clockwise check (signed area > 0), fix any block with the other orientation
    P = pts2[quads]
    area = 0.5 * np.sum(P[:, :, 0] * np.roll(P[:, :, 1], -1, axis=1) - np.roll(P[:, :, 0], -1, axis=1) * P[:, :, 1],
                        axis=1)
    quads[area < 0] = quads[area < 0][:, ::-1]
    if jitter > 0.0:
        n = len(pts2)
        e = np.concatenate([quads[:, [0, 1]], quads[:, [1, 2]], quads[:, [2, 3]], quads[:, [3, 0]]])
        le = np.linalg.norm(pts2[e[:, 0]] - pts2[e[:, 1]], axis=1)
        hmin = np.full(n, np.inf)
        np.minimum.at(hmin, e[:, 0], le)
        np.minimum.at(hmin, e[:, 1], le)
        rr = np.hypot(pts2[:, 0] - cx, pts2[:, 1] - cy)
        eps = 1e-9
        fixed = ((pts2[:, 0] < eps) | (pts2[:, 0] > length - eps) | (pts2[:, 1] < eps) |
                 (pts2[:, 1] > height - eps) | (np.abs(rr - r0) < 1e-7))
        rng = np.random.default_rng(seed)
        d = rng.uniform(-1.0, 1.0, size=(n, 2)) * (jitter * hmin)[:, None]
        d[fixed] = 0.0
        pts2 = pts2 + d
    nn = len(pts2)
    pts3 = np.concatenate([np.column_stack([pts2, np.zeros(nn)]), np.column_stack([pts2, np.full(nn, dz)])])
    hexes = np.concatenate([quads, quads + nn], axis=1)
    if prisms:
        # counter-clockwise quads -> two counter-clockwise triangles -> two wedges in place
        far = np.concatenate(far_list)
        flat, types = _cells_with_prisms(hexes, far)
        return UnstructuredGrid(flat, types, pts3), {"cylinder": (cx, cy, r0)}
    cells = np.hstack([np.full((len(hexes), 1), 8), hexes]).ravel()
    return UnstructuredGrid(cells, np.full(len(hexes), HEXAHEDRON), pts3), {"cylinder": (cx, cy, r0)}


def define_cylinder_group(m: Mesh, cylinder, name="cylinder", tol=1e-6):
    """Group the boundary faces on the cylinder surface: in-plane normal (not the front or
    back face of a cell) and centroid on the circle."""
    cx, cy, r0 = cylinder
    fp, cp = m.face_properties, m.cell_properties
    b = fp.boundary_face_ids
    c = m._geometry64["face_centroid"][b]
    nz = cp.normal[fp.adjacent_cells[b, 0], fp.cell_face_index[b, 0], 2]
    rr = np.hypot(c[:, 0] - cx, c[:, 1] - cy)
    ids = b[(np.abs(nz) < 0.5) & (np.abs(rr - r0) < r0 * 0.05 + tol)]
    m.add_group(name, ids, "face")
    return ids
