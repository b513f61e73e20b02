"""The int16 column-offset table of the ELL matrix (wcfd_mesh.ell_dcol): present exactly
when every |column - row| fits in int16, and equal to the columns minus their rows."""
import numpy as np

from tests.cases import cavity3d_mesh, cavity_mesh


def test_offsets_equal_columns_minus_rows():
    from warpcfd_gb300.FV.geometry import build_geometry

    for m in (cavity_mesh(12, jitter=0.1, seed=2), cavity3d_mesh(6)):
        g = build_geometry(m)
        d = g["ell_dcol"]
        assert d is not None and d.dtype == np.int16 and d.shape == g["ell_col"].shape
        rows = np.arange(g["n_cells"])[None, :]
        assert np.array_equal(d.astype(np.int64) + rows, g["ell_col"].astype(np.int64))


def test_offsets_absent_when_they_do_not_fit():
    from warpcfd_gb300.FV.geometry import ell_offsets

    C = 40000
    col = np.tile(np.arange(C, dtype=np.int32), (4, 1))
    col[1, 5] = 5 + 32767
    assert ell_offsets(col) is not None
    col[2, 7] = 7 + 32768
    assert ell_offsets(col) is None
    col[2, 7] = 7
    col[0, 39999] = 39999 - 32768
    assert ell_offsets(col) is None
    assert ell_offsets(np.zeros((1, 0), dtype=np.int32)) is None
