"""Failure detection on the GPU without a fault: the grid barrier of the cooperative Krylov
kernels is checked for correct sums, and a wait that nothing satisfies (one block never
arrives) runs out after its bounded limit and comes back as WCFD_BARRIER_TIMEOUT with the
context still usable."""
import ctypes as ct
import time

import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib_ready():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from warpcfd_gb300.build import build_library
    build_library()


def _check(skip, phases):
    from warpcfd_gb300 import _lib
    res = (ct.c_int32 * 3)()
    _lib.check(_lib.load().wcfd_grid_barrier_check(skip, phases, res, None))
    return list(res)


def test_grid_barrier_sums_are_exact():
    status, bad, blocks = _check(-1, 2000)
    assert (status, bad) == (0, 0)
    assert blocks >= torch.cuda.get_device_properties(0).multi_processor_count


def test_grid_barrier_wait_runs_out_and_context_survives():
    from warpcfd_gb300 import _lib
    _, _, blocks = _check(-1, 1)
    t0 = time.perf_counter()
    status, bad, _ = _check(blocks - 1, 5)
    elapsed = time.perf_counter() - t0
    assert status == _lib.WCFD_BARRIER_TIMEOUT and bad == 0
    assert 1.0 < elapsed < 30.0
    # the context is still usable: a clean check and a device computation afterwards
    assert _check(-1, 10)[:2] == [0, 0]
    x = torch.arange(1000, device="cuda", dtype=torch.float32)
    assert float(x.sum()) == 499500.0


def test_device_mesh_check_passes_valid_meshes_and_reports_corrupt_ones():
    """wcfd_check_mesh: zero violations on hex, mixed, tetrahedral and one-cell meshes (it
    runs in every finalize); each kind of corrupt index array is counted and reported as a
    status, with no access outside the arrays (indices are checked before they are used)."""
    import ctypes as ct

    from tests.cases import cavity_bc, cavity_mesh, mixed_cavity3d_mesh, tet_cavity3d_mesh
    from tests.gpu_helpers import make_pair
    from warpcfd_gb300 import _lib
    from warpcfd_gb300.preprocess import Mesh, create_2D_grid, define_boundary_walls

    one = Mesh(create_2D_grid((0, 0, 0), 1, 1, 1.0, 1.0, 0.1))
    define_boundary_walls(one)
    for m in (cavity_mesh(8, jitter=0.1, seed=2), mixed_cavity3d_mesh(5), tet_cavity3d_mesh(3), one):
        model, _, _ = make_pair(m, cavity_bc)
        assert model.check_mesh() == [0, 0, 0, 0, 0]

    model, _, _ = make_pair(cavity_mesh(6), cavity_bc)
    g = model._geo
    lib = _lib.load()

    def counts_with(**swap):
        ms = model.mesh_struct()
        keep = []
        for name, arr in swap.items():
            keep.append(arr)
            setattr(ms, name, arr.data_ptr())
        out = (ct.c_int32 * 5)()
        rc = lib.wcfd_check_mesh(ct.byref(ms), out, None)
        return rc, list(out)

    owner = g["face_owner"].clone()
    owner[3] = model.num_cells + 7
    rc, c = counts_with(face_owner=owner)
    assert rc == _lib.WCFD_ERR_ARGUMENT and c[0] == 1
    col = g["ell_col"].clone()
    col.view(-1)[5] = -2
    rc, c = counts_with(ell_col=col)
    assert rc == _lib.WCFD_ERR_ARGUMENT and c[4] == 1
    slot = g["cell_slot"].clone()
    w = slot.view(-1, 4)[:, 3].view(torch.int32)
    w[0] = 10 ** 8                       # a face id past the end
    w[1] = int(w[2])                     # a face that does not border this cell
    rc, c = counts_with(cell_slot=slot)
    assert rc == _lib.WCFD_ERR_ARGUMENT and c[2] == 1 and c[3] >= 1
    assert "slot/face mismatches" in lib.wcfd_mesh_last_error().decode()
