"""Mesh preprocessing: vectorised pass vs the loop restatement of the reference's pass,
plus geometric identities."""
import numpy as np
import pytest

from oracle.mesh_ref import reference_mesh_properties
from tests.cases import cavity3d_mesh, cavity_mesh, channel_mesh
from warpcfd_gb300.preprocess import Mesh, create_2D_grid, define_boundary_walls


@pytest.mark.parametrize("make", [lambda: cavity_mesh(5), lambda: cavity_mesh(6, jitter=0.1, seed=3),
                                  lambda: cavity3d_mesh(4, jitter=0.1, seed=1), lambda: channel_mesh(7, 3)])
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
        create_2D_grid((0, 0, 0), 2, 2, 1, 1, 0.1, element_type="wedge")
    m = Mesh(g)
    define_boundary_walls(m)
    with pytest.raises(AssertionError):
        m.add_group("+X", [0], "face")
