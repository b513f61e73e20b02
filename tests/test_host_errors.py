"""The drop-in's host-side error behaviour follows the reference's (boundary.py:31-121):
the same exception types for an unknown group, a non-boundary face, a call without fields,
an unsupported id type and faces left without a condition; per-face value arrays land in
the group's boundary-row order."""
import numpy as np
import pytest

from tests.cases import FIELDS, cavity_mesh
from warpcfd_gb300.FV.boundary import Boundary


def _boundary(m):
    return Boundary(FIELDS, m.groups, m.face_properties.boundary_face_ids)


def test_boundary_errors_match_the_reference():
    m = cavity_mesh(4)
    b = _boundary(m)
    with pytest.raises(AssertionError, match="group name does not exist"):
        b.no_slip_wall("+W")
    internal = int(m.face_properties.internal_face_ids[0])
    with pytest.raises(AssertionError, match="not an external face"):
        b.fixed_BC([internal], u=1.0)
    with pytest.raises(AssertionError, match="some sort of output variable"):
        b.fixed_BC("-X")
    with pytest.raises(ValueError, match="face_ids can be type"):
        b.fixed_BC(1.5, u=1.0)
    b.no_slip_wall("-X")
    with pytest.raises(ValueError, match="have not been assigned a boundary condition"):
        b.check()
    for g in ("+X", "-Y", "+Y", "+Z", "-Z"):
        b.slip_wall(g)
    b.check()


def test_per_face_values_follow_the_group_order():
    m = cavity_mesh(4)
    b = _boundary(m)
    ids = np.asarray(m.groups["+Y"].ids)
    vals = np.arange(len(ids), dtype=np.float64) + 1.0
    b.velocity_BC("+Y", u=vals, v=0.0, w=0.0)
    rows = np.where(np.isin(m.face_properties.boundary_face_ids, ids))[0]
    # rows in boundary order, values assigned to them in that order
    assert np.array_equal(b.boundary_values[rows, 0], vals)
    assert np.all(b.boundary_type[rows, 0] == 1)


def test_boundary_rows_lookup_equals_set_membership():
    """The face-id lookup set_value uses gives the rows np.where(np.isin(boundary_ids,
    face_ids)) gives (boundary.py:40-45), duplicates and non-boundary ids included."""
    import numpy as np

    from warpcfd_gb300.FV.boundary.boundary import Boundary

    rng = np.random.default_rng(0)
    for t in range(100):
        bids = np.sort(rng.choice(5000, size=rng.integers(1, 800), replace=False)).astype(np.int32)
        b = Boundary({"u": None}, {}, bids)
        f = rng.choice(bids, size=rng.integers(1, 300))
        if t % 3 == 0:
            f = np.concatenate([f, rng.integers(-3, 6000, size=5)])
        rows, ok = b._rows(f)
        assert np.array_equal(rows, np.where(np.isin(bids, f))[0])
        assert ok == bool(np.all(np.isin(f, bids)))
