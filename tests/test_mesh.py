"""Mesh preprocessing: vectorised pass vs the loop restatement of the reference's pass,
plus geometric identities."""
import numpy as np
import pytest

from oracle.mesh_ref import reference_mesh_properties
from tests.cases import cavity3d_mesh, cavity_mesh, channel_mesh
from warpcfd_gb300.preprocess import Mesh, create_2D_grid, create_3D_grid, define_boundary_walls


@pytest.mark.parametrize("make", [lambda: cavity_mesh(5), lambda: cavity_mesh(6, jitter=0.1, seed=3),
                                  lambda: cavity3d_mesh(4, jitter=0.1, seed=1), lambda: channel_mesh(7, 3),
                                  lambda: Mesh(create_2D_grid((0, 0, 0), 5, 4, 1.0, 1.0, 0.1,
                                                              element_type="wedge", jitter=0.1, seed=2)),
                                  lambda: Mesh(create_3D_grid((0, 0, 0), 3, 3, 2, 1.0, 1.0, 0.5, element_type="tetra",
                                                              jitter=0.15, seed=4))])
def test_matches_reference_loop(make):
    m = make()
    ref = reference_mesh_properties(m.nodes.astype(np.float64), m.cells)
    fp, cp = m.face_properties, m.cell_properties
    np.testing.assert_array_equal(fp.unique_faces, ref["unique_faces"])
    np.testing.assert_array_equal(cp.faces, ref["cell_faces"])
    np.testing.assert_array_equal(fp.adjacent_cells, ref["adjacent"])
    np.testing.assert_array_equal(fp.cell_face_index, ref["cell_face_index"])
    np.testing.assert_array_equal(fp.is_boundary, ref["is_boundary"])
    np.testing.assert_array_equal(cp.neighbors, ref["neighbors"])
    np.testing.assert_array_equal(cp.face_side, ref["face_side"])
    np.testing.assert_array_equal(cp.nnz_per_cell, ref["nnz_per_cell"])
    np.testing.assert_array_equal(cp.face_offset_index, ref["face_offset_index"])
    np.testing.assert_array_equal(fp.boundary_face_ids, ref["boundary_face_ids"])
    np.testing.assert_array_equal(fp.internal_face_ids, ref["internal_face_ids"])
    np.testing.assert_allclose(cp.normal, ref["normal"], atol=1e-6)
    np.testing.assert_allclose(cp.area, ref["area"], rtol=1e-6)
    np.testing.assert_allclose(cp.cell_centroid_to_face_centroid, ref["to_face"], atol=1e-6)
    d = fp.distance.astype(np.float64)
    np.testing.assert_allclose(d, ref["distance"], atol=1e-6)


def test_benchmark_sizes():
    m = cavity_mesh(64)
    assert (m.num_cells, m.num_faces, len(m.face_properties.internal_face_ids)) == (4096, 16512, 8064)
    assert int(m.cell_properties.nnz_per_cell.sum()) == 20224
    m = channel_mesh(400, 80)
    assert (m.num_cells, len(m.face_properties.internal_face_ids), m.face_properties.num_boundary_faces) == \
        (32000, 63520, 64960)
    assert int(m.cell_properties.nnz_per_cell.sum()) == 159040


@pytest.mark.parametrize("jitter", [0.0, 0.1])
def test_closed_cells_and_volume(jitter):
    m = cavity3d_mesh(5, jitter=jitter, seed=7)
    g = m._geometry64
    s = (g["normal"] * g["area"][..., None]).sum(axis=1)
    assert np.abs(s).max() < 1e-12
    assert abs(g["volume"].sum() - 1.0) < 1e-12
    assert (g["volume"] > 0).all()


def test_owner_is_lower_and_normals_outward():
    m = cavity_mesh(6, jitter=0.1, seed=2)
    fp, cp = m.face_properties, m.cell_properties
    ii = fp.internal_face_ids
    assert (fp.adjacent_cells[ii, 0] < fp.adjacent_cells[ii, 1]).all()
    # owner normal points from owner to neighbour
    P, N = fp.adjacent_cells[ii, 0], fp.adjacent_cells[ii, 1]
    n = cp.normal[P, fp.cell_face_index[ii, 0]]
    d = m.cell_centroids[N] - m.cell_centroids[P]
    assert (np.sum(n * d, axis=1) > 0).all()
    # the two sides see opposite normals
    n2 = cp.normal[N, fp.cell_face_index[ii, 1]]
    np.testing.assert_allclose(n, -n2, atol=1e-6)


def test_walls():
    m = cavity_mesh(8)
    sizes = {k: len(v.ids) for k, v in m.groups.items()}
    assert sizes == {"+X": 8, "-X": 8, "+Y": 8, "-Y": 8, "+Z": 64, "-Z": 64}
    allb = np.concatenate([v.ids for v in m.groups.values()])
    assert sorted(allb.tolist()) == sorted(m.face_properties.boundary_face_ids.tolist())


def test_rejects_mixed_and_bad_input():
    class G:
        points = np.zeros((4, 3))
        cells_dict = {12: np.zeros((1, 8), dtype=int), 13: np.zeros((1, 6), dtype=int)}
    with pytest.raises(AssertionError):
        Mesh(G())
    g = create_2D_grid((0, 0, 0), 2, 2, 1, 1, 0.1)
    with pytest.raises(NotImplementedError):
        create_2D_grid((0, 0, 0), 2, 2, 1, 1, 0.1, element_type="tet")
    m = Mesh(g)
    define_boundary_walls(m)
    with pytest.raises(AssertionError):
        m.add_group("+X", [0], "face")


@pytest.mark.parametrize("make", [
    lambda: create_2D_grid((0, 0, 0), 6, 5, 1.0, 1.0, 0.1, element_type="mixed", jitter=0.1, seed=4),
    lambda: create_3D_grid((0, 0, 0), 5, 4, 3, 1.0, 0.8, 0.6, prism_fraction=0.4, seed=3)])
def test_mixed_hex_prism_mesh(make):
    """Mixed meshes (an extension: the reference takes one cell type): null slots past a
    wedge's five faces, outward normals, closed cells, matched internal faces, the
    domain's volume, triangles numbered before quads, and the hexes' own faces."""
    g = make()
    m = Mesh(g)
    assert m.cellType == ("MIXED", 0)
    fp, cp, g64 = m.face_properties, m.cell_properties, m._geometry64
    types = m.cell_types
    assert cp.faces.shape[1] == 6
    valid = cp.slot_valid
    assert np.array_equal(valid.sum(axis=1), np.where(types == 12, 6, 5))
    assert np.all(cp.faces[~valid] == -1) and np.all(cp.neighbors[~valid] == -1)
    assert np.all(cp.area[~valid] == 0) and np.all(cp.face_offset_index[~valid] == 0)
    # outward, closed
    d = np.einsum("cfk,cfk->cf", g64["normal"], g64["to_face"])
    assert d[valid].min() > 0
    assert np.abs((g64["normal"] * g64["area"][..., None]).sum(axis=1)).max() < 1e-12
    # every internal face seen from both sides with opposite normals and equal areas
    ii = fp.internal_face_ids
    P, N = fp.adjacent_cells[ii, 0], fp.adjacent_cells[ii, 1]
    sP, sN = fp.cell_face_index[ii, 0], fp.cell_face_index[ii, 1]
    assert np.all(P < N)
    assert np.array_equal(cp.faces[P, sP], ii) and np.array_equal(cp.faces[N, sN], ii)
    assert np.abs(g64["normal"][P, sP] + g64["normal"][N, sN]).max() < 1e-12
    assert np.array_equal(cp.neighbors[P, sP], N) and np.array_equal(cp.neighbors[N, sN], P)
    # boundary slots are exactly the valid slots without a neighbour
    b = fp.boundary_face_ids
    assert len(b) == int((valid & (cp.neighbors == -1)).sum())
    lo = g.points.min(axis=0)
    hi = g.points.max(axis=0)
    assert abs(g64["volume"].sum() - np.prod(hi - lo)) < 1e-12
    # triangles first, each node-count set in lexicographic order of sorted node ids
    npf = fp.num_nodes
    nt = int((npf == 3).sum())
    assert np.all(npf[:nt] == 3) and np.all(npf[nt:] == 4)
    for lo_, hi_ in ((0, nt), (nt, len(npf))):
        rows = fp.unique_faces[lo_:hi_, :int(npf[lo_])].astype(np.int64)
        keys = [tuple(r) for r in rows]
        assert keys == sorted(keys) and len(set(keys)) == len(keys)
    # a hex keeps its own face table: slot 0 is its bottom quad (3, 2, 1, 0)
    h = int(np.nonzero(types == 12)[0][0])
    assert sorted(fp.unique_faces[cp.faces[h, 0]].tolist()) == sorted(m.cells[h, [3, 2, 1, 0]].tolist())
