"""The mesh pass on the GPU (libwcfd wcfd_mesh_*) against the host pass: topology bit for
bit, float64 geometry bit for bit where the host pass's order of operations is known
(fan triangulation, node means), the cell volume to rounding."""
import numpy as np
import pytest
import torch

from warpcfd_gb300.preprocess import Mesh, create_2D_grid, create_3D_grid, create_cylinder_channel_grid

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib_ready():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from warpcfd_gb300.build import build_library
    build_library()


GRIDS = {
    "hex2d_jitter": lambda: create_2D_grid((0, 0, 0), 17, 11, 1.0, 0.7, 0.1, jitter=0.15, seed=2),
    "hex3d_jitter": lambda: create_3D_grid((0, 0, 0), 9, 7, 5, 1.0, 0.8, 0.6, jitter=0.2, seed=3),
    "prism2d": lambda: create_2D_grid((0, 0, 0), 12, 9, 2.0, 1.0, 0.1, element_type="wedge", jitter=0.1, seed=1),
    "mixed2d": lambda: create_2D_grid((0, 0, 0), 14, 6, 3.0, 1.0, 0.1, element_type="mixed"),
    "mixed3d": lambda: create_3D_grid((0, 0, 0), 8, 6, 5, 1.0, 1.0, 1.0, prism_fraction=0.4, seed=7),
    "tetra3d_jitter": lambda: create_3D_grid((0, 0, 0), 6, 5, 4, 1.0, 1.0, 1.0, element_type="tetra", jitter=0.2, seed=8),
    "cylinder": lambda: create_cylinder_channel_grid(scale=0.5)[0],
    "single_hex": lambda: create_3D_grid((0, 0, 0), 1, 1, 1, 1.0, 1.0, 1.0),
    "single_hex_as_tets": lambda: create_3D_grid((0, 0, 0), 1, 1, 1, 1.0, 1.0, 1.0, element_type="tetra"),
}

INT_FACE = ("unique_faces", "adjacent_cells", "cell_face_index", "is_boundary", "boundary_face_ids",
            "internal_face_ids", "num_nodes")
INT_CELL = ("faces", "neighbors", "face_side", "nnz_per_cell", "face_offset_index")


@pytest.mark.parametrize("name", list(GRIDS))
def test_device_mesh_pass_matches_host_pass(name):
    g = GRIDS[name]()
    h = Mesh(g)
    d = Mesh(g, device="cuda")
    for k in INT_FACE:
        np.testing.assert_array_equal(getattr(d.face_properties, k), getattr(h.face_properties, k), err_msg=k)
    for k in INT_CELL:
        np.testing.assert_array_equal(getattr(d.cell_properties, k), getattr(h.cell_properties, k), err_msg=k)
    for k in ("area", "normal", "to_face", "face_centroid"):
        np.testing.assert_array_equal(d._geometry64[k], h._geometry64[k], err_msg=k)
    np.testing.assert_array_equal(d._centroids64, h._centroids64)
    np.testing.assert_allclose(d._geometry64["volume"], h._geometry64["volume"], rtol=1e-13)
    np.testing.assert_array_equal(d.face_properties.distance, h.face_properties.distance)


def test_device_mesh_pass_reports_bad_cells():
    """A node id out of range comes back as an error, not a fault: the kernels check ids
    before they use them."""
    from warpcfd_gb300 import _lib
    g = create_3D_grid((0, 0, 0), 3, 3, 3, 1.0, 1.0, 1.0)
    g.cells = g.cells.copy()
    g.cells[1 + 3] = 10_000  # a node of the first hex
    g.cells_dict = {12: g.cells.reshape(-1, 9)[:, 1:]}
    with pytest.raises(_lib.WcfdError, match="out of range"):
        Mesh(g, device="cuda")
