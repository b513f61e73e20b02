"""Boundary-condition registry (warp_cfd/FV/boundary/boundary.py:5-121).

One row per boundary face (in ``boundary_ids`` order) and one column per field
(u, v, w, p).  Type 1 = fixed value (Dirichlet), 2 = fixed normal gradient (Neumann).
Values may be a scalar or a per-face array of the selected faces' length
(boundary.py:31-45).  ``finalize`` checks completeness and moves the table to the
device as int8/float tensors.
"""
from __future__ import annotations

import numpy as np

DIRICHLET = 1
NEUMANN = 2


class Boundary:
    def __init__(self, fields, groups, boundary_ids, face_areas=None, face_normals=None, face_centroids=None,
                 float_type=np.float32) -> None:
        self.fields = fields
        self.num_outputs = len(list(self.fields.keys()))
        self.groups = groups
        self.boundary_ids = np.asarray(boundary_ids)
        self.boundary_values = np.zeros((len(self.boundary_ids), self.num_outputs), dtype=np.float64)
        self.boundary_type = np.zeros(self.boundary_values.shape, dtype=np.uint8)
        self.float_dtype = float_type
        self._boundary_types = {"dirichlet": DIRICHLET, "vonNeumann": NEUMANN}
        self.finalized = False
        self._row_of = None   # face id -> boundary row (-1: not a boundary face), built on first use

    def _rows(self, face_ids):
        """(rows, all_boundary): the boundary rows of ``face_ids`` in boundary order, each
        once -- the rows np.where(np.isin(boundary_ids, face_ids)) gives -- and whether every
        id is a boundary face, by a face-id lookup table instead of sorted set membership."""
        B = len(self.boundary_ids)
        if self._row_of is None:
            bids = self.boundary_ids.astype(np.int64)
            self._row_of = np.full(int(bids.max()) + 1 if B else 0, -1, dtype=np.int64)
            self._row_of[bids] = np.arange(B)
        f = np.asarray(face_ids).astype(np.int64, copy=False).reshape(-1)
        inside = (f >= 0) & (f < self._row_of.shape[0])
        r = self._row_of[f[inside]]
        all_boundary = bool(inside.all()) and bool((r >= 0).all())
        mask = np.zeros(B, dtype=bool)
        mask[r[r >= 0]] = True
        return np.flatnonzero(mask), all_boundary

    def set_value(self, face_ids, boundary_type="dirchlet", **output_vars):
        face_ids = self.get_face_id_array(face_ids)
        rows, all_boundary = self._rows(face_ids)
        if not all_boundary:
            raise AssertionError("One or more of the provided face id is not an external face valid for "
                                 "applying boundary conditions")
        if not output_vars:
            raise AssertionError("You must specify some sort of output variable")
        # rows in boundary order; a per-face array is assigned to them in that order, as
        # boundary.py:40-45 does (np.where(np.isin(self.boundary_ids, face_ids)))
        for output_name, value in output_vars.items():
            output = self.fields[output_name]
            self.boundary_values[rows, output.index] = np.asarray(value, dtype=np.float64)
            self.boundary_type[rows, output.index] = self._boundary_types[boundary_type]

    def get_face_id_array(self, face_ids):
        if isinstance(face_ids, str):
            assert face_ids in list(self.groups.keys()), "Specified group name does not exist"
            return np.asarray(self.groups[face_ids].ids)
        elif isinstance(face_ids, (int, np.integer, list, tuple, np.ndarray)):
            if not isinstance(face_ids, np.ndarray):
                return np.array(face_ids, np.int32).reshape(-1)
            return face_ids
        raise ValueError(f"face_ids can be type string,int,list,tuple, or np.ndarray got {type(face_ids)} instead")

    def gradient_BC(self, face_ids, **output_vars):
        """Fixed normal gradient (type 2) for the named fields."""
        self.set_value(face_ids, **output_vars, boundary_type="vonNeumann")

    def fixed_BC(self, face_ids, **output_vars):
        """Fixed value (type 1) for the named fields."""
        self.set_value(face_ids, **output_vars, boundary_type="dirichlet")

    def velocity_BC(self, face_ids, u, v, w):
        """Fixed u, v, w and zero normal gradient of p."""
        self.fixed_BC(face_ids, u=u, v=v, w=w)
        self.gradient_BC(face_ids, p=0.0)

    def pressure_BC(self, face_ids, p, backflow=None):
        """Fixed p and zero normal gradient of u, v, w."""
        self.fixed_BC(face_ids, p=p)
        self.gradient_BC(face_ids, u=0.0, v=0.0, w=0.0)

    def mass_flow_BC(self, face_ids, mass_flow, inlet=True):
        raise ValueError("not yet implemented")

    def no_slip_wall(self, face_ids):
        """u = v = w = 0 and zero normal gradient of p."""
        self.fixed_BC(face_ids, u=0.0, v=0.0, w=0.0)
        self.gradient_BC(face_ids, p=0.0)

    def slip_wall(self, face_ids):
        """Zero normal gradient of u, v, w and p."""
        self.gradient_BC(face_ids, u=0.0, v=0.0, w=0.0, p=0.0)

    def check(self):
        """Completeness checks of boundary.py:108-121."""
        if np.any(self.boundary_type < 1):
            missing = self.boundary_ids[(self.boundary_type < 1).all(axis=1)]
            raise ValueError(f"The following faces have not been assigned a boundary condition: {missing}")
        if np.any(self.boundary_type > 3):
            raise ValueError("Somehow you have a boundary type with a value of 3. Only 1 and 2 arw allowed")

    def finalize(self):
        self.check()
        self.finalized = True
