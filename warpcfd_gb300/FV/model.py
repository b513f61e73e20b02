"""FVM: the model state and field operators, with the API of warp_cfd.FV.FVM
(warp_cfd/FV/model.py:51-349).

Fields are torch tensors on one CUDA device; every operator runs a libwcfd kernel on
the current torch stream.  Layouts match the reference's arrays: cell_values (C,4)
u,v,w,p; cell_gradients (C,4,3); face_values (K,4); face_gradients (K,4);
mass_fluxes (K,), with the reference's face numbering.
"""
from __future__ import annotations

import ctypes as ct

import numpy as np
import torch

from .. import _lib
from ..material import Material
from .boundary import Boundary
from .convergence import Convergence
from .field import Field
from .geometry import build_geometry


class CFD_settings:
    """Declared settings (model.py:40-48); kept as API surface."""
    steady_state: bool = True
    velocity_face_interpolation: str = "central difference"
    interpolation_schemes = {"central difference": 0, "upwind": 1, "upwind-linear": 2}


def _torch_float(dtype):
    if dtype in (None, torch.float32, np.float32, "float32", "fp32"):
        return torch.float32
    name = getattr(dtype, "__name__", str(dtype))
    if "32" in name:
        return torch.float32
    raise NotImplementedError("the GB300 path computes fields in float32 (fp64 is kept for Krylov reductions)")


def _ptr(t):
    return ct.c_void_p(t.data_ptr()) if t is not None else ct.c_void_p(0)


def _stream():
    return ct.c_void_p(torch.cuda.current_stream().cuda_stream)


class FVM:
    """Finite-volume model of one mesh (model.py:51-116)."""

    def __init__(self, mesh, output_variables=None, float_dtype=torch.float32, int_dtype=torch.int32, device=None):
        self.material = Material()
        self.dimension = mesh.dimension
        self.float_dtype = _torch_float(float_dtype)
        self.int_dtype = torch.int32
        self.mesh = mesh
        self.settings = CFD_settings()
        self.Convergence = Convergence()
        self.skew_correction = True
        self.face_properties = mesh.face_properties
        self.cell_properties = mesh.cell_properties
        self.node_properties = mesh.nodes
        self.input_variables = ["x", "y", "z", "t"]
        self.output_variables = list(output_variables) if output_variables is not None else ["u", "v", "w", "p"]
        if self.output_variables != ["u", "v", "w", "p"]:
            raise NotImplementedError("the incompressible kernels carry the fields u, v, w, p in that order")
        self.fields = {name: Field(name, i) for i, name in enumerate(self.output_variables)}
        self.boundary = Boundary(self.fields, mesh.groups, boundary_ids=self.face_properties.boundary_face_ids)
        self.vars_mapping = {var: i for i, var in enumerate(self.output_variables)}
        self.num_outputs = len(self.output_variables)
        self.num_nodes = mesh.nodes.shape[0]
        self.num_cells = mesh.cells.shape[0]
        self.num_faces = mesh.face_properties.unique_faces.shape[0]
        self.nodes_per_cell = mesh.cells.shape[-1]
        self.faces_per_cell = self.cell_properties.faces_per_cell
        self.nodes_per_face = self.cell_properties.nodes_per_face
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device()
                                                                                  if torch.cuda.is_available() else 0)
        self.reference_pressure_cell_id = None
        self.reference_pressure = 0.0
        self.finalized = False
        self._geo = None
        self._gdiff_corrected = None

    # ------------------------------------------------------------------ finalize
    def finalize(self):
        """Check BCs, move geometry and BC tables to the device, allocate the fields
        (model.py:121-139)."""
        if self.finalized:
            return
        _lib.load()
        self.boundary.finalize()
        dev = self.device
        # the geometry is read-only on the device: models of the same mesh share one copy
        cache = self.mesh.__dict__.setdefault("_device_geometry", {})
        key = str(torch.device(dev))
        fresh = key not in cache
        if fresh:
            geo = build_geometry(self.mesh, correction=False)
            cache[key] = (geo, {k: (torch.from_numpy(np.ascontiguousarray(v)).to(dev) if isinstance(v, np.ndarray)
                                    else v) for k, v in geo.items()})
        self._geo_host, self._geo = cache[key]
        if fresh:
            self.check_mesh()
        self.boundary_type = torch.from_numpy(self.boundary.boundary_type.copy()).to(dev)
        self.boundary_value = torch.from_numpy(self.boundary.boundary_values.astype(np.float32)).to(dev)
        self.boundary_ids = self._geo["boundary_face"]
        self.init_global_arrays()
        self.finalized = True

    def check_mesh(self):
        """Bounds and consistency check of the device geometry's index arrays
        (wcfd_check_mesh); raises WcfdError naming the violations.  Run once per mesh and
        device by finalize()."""
        import ctypes as ct
        counts = (ct.c_int32 * 5)()
        lib = _lib.load()
        rc = lib.wcfd_check_mesh(ct.byref(self.mesh_struct()), counts,
                                 ct.c_void_p(torch.cuda.current_stream(self.device).cuda_stream))
        if rc != _lib.WCFD_OK:
            raise _lib.WcfdError(rc, lib.wcfd_mesh_last_error().decode(errors="replace"))
        return list(counts)

    def init_global_arrays(self):
        C, K, dev, T = self.num_cells, self.num_faces, self.device, self.float_dtype
        self.cell_values = torch.zeros((C, 4), dtype=T, device=dev)
        self.cell_gradients = torch.zeros((C, 4, 3), dtype=T, device=dev)
        self.face_values = torch.zeros((K, 4), dtype=T, device=dev)
        self.face_gradients = torch.zeros((K, 4), dtype=T, device=dev)
        self.mass_fluxes = torch.zeros(K, dtype=T, device=dev)

    def mesh_struct(self, correction: bool = False) -> _lib.Mesh_t:
        """The C struct view of the device geometry (gdiff with or without the
        non-orthogonal |n1| factor)."""
        g = self._geo
        gdiff = g["face_gdiff"]
        if correction:
            if self._gdiff_corrected is None:
                gc = build_geometry(self.mesh, correction=True)["face_gdiff"]
                self._gdiff_corrected = torch.from_numpy(gc).to(self.device)
            gdiff = self._gdiff_corrected
        return _lib.Mesh_t(
            g["n_cells"], g["n_faces"], g["n_bfaces"], g["faces_per_cell"], g["ell_width"], 0,
            g["face_owner"].data_ptr(), g["face_nbr"].data_ptr(), g["face_brow"].data_ptr(),
            g["face_interp"].data_ptr(), g["face_normal"].data_ptr(), gdiff.data_ptr(),
            g["face_rpf"].data_ptr(), g["cell_slot"].data_ptr(), g["cell_volume"].data_ptr(),
            g["ell_col"].data_ptr(), g["boundary_face"].data_ptr(), g["face_dvec"].data_ptr(),
            g["ell_dcol"].data_ptr() if g.get("ell_dcol") is not None else None)

    def bc_struct(self) -> _lib.BC_t:
        return _lib.BC_t(self.boundary_type.data_ptr(), self.boundary_value.data_ptr())

    def state_struct(self) -> _lib.State_t:
        return _lib.State_t(self.cell_values.data_ptr(), self.cell_gradients.data_ptr(),
                            self.face_values.data_ptr(), self.face_gradients.data_ptr(),
                            self.mass_fluxes.data_ptr())

    def _need_final(self):
        if not self.finalized:
            raise ValueError("Please call method model.finalize() first")

    # ------------------------------------------------------------------ API
    def set_initial_conditions(self, IC, output_indices=None):
        """Copy IC (C, n) into cell_values (model.py:143-148, conditions.py:28-32)."""
        self._need_final()
        IC = torch.as_tensor(IC, dtype=self.float_dtype, device=self.device)
        idx = list(range(IC.shape[-1])) if output_indices is None else self._index_list(output_indices)
        for i in idx:
            self.cell_values[:, i].copy_(IC[:, i])

    def set_reference_pressure(self, cell_id: int, value: float = 0.0):
        self.reference_pressure_cell_id = cell_id
        self.reference_pressure = float(value)

    def _index_list(self, output_indices):
        if output_indices is None:
            return list(range(self.num_outputs))
        if isinstance(output_indices, (int, np.integer)):
            return [int(output_indices)]
        if isinstance(output_indices, str):
            assert output_indices in self.output_variables, \
                "output indices type str was not found in model's list of output variables"
            return [self.fields[output_indices].index]
        out = []
        for o in output_indices:
            out.append(self.fields[o].index if isinstance(o, str) else int(o))
        return out

    def get_output_indices(self, output_indices):
        """Field selection as a bit mask u=1, v=2, w=4, p=8 (model.py:193-204)."""
        mask = 0
        for i in self._index_list(output_indices):
            mask |= 1 << i
        return mask

    def set_boundary_conditions(self):
        self._need_final()
        _lib.call("wcfd_set_boundary_conditions", ct.byref(self.mesh_struct()), self.bc_struct(),
                  self.state_struct(), _stream())

    def face_interpolation(self, output_indices=None, upwind=False):
        self._need_final()
        _lib.call("wcfd_face_interpolation", ct.byref(self.mesh_struct()), self.bc_struct(), self.state_struct(),
                  self.get_output_indices(output_indices), int(self.skew_correction), int(bool(upwind)), _stream())

    def calculate_gradients(self, output_indices=None):
        self._need_final()
        _lib.call("wcfd_calculate_gradients", ct.byref(self.mesh_struct()), self.state_struct(),
                  self.get_output_indices(output_indices), _stream())

    def get_gradient(self, output_index, coeff=1.0):
        """Copy of coeff * grad(field) as (C,3) (model.py:242-254)."""
        if isinstance(output_index, str):
            output_index = self.fields[output_index].index
        g = self.cell_gradients[:, output_index, :]
        if isinstance(coeff, (float, int)):
            return (float(coeff) * g).contiguous()
        return (coeff.reshape(-1, 1) * g).contiguous()

    def relax(self, new_value, alpha, output_index):
        """cell_values[:,o] = alpha new + (1 - alpha) old (model.py:256-262, :381-384)."""
        if isinstance(output_index, str):
            output_index = self.fields[output_index].index
        col = self.cell_values[:, output_index]
        col.copy_(alpha * new_value.reshape(-1) + (1.0 - alpha) * col)

    def calculate_mass_flux(self):
        self._need_final()
        _lib.call("wcfd_calculate_mass_flux", ct.byref(self.mesh_struct()), self.state_struct(), _stream())

    def divFlux(self, arr=None):
        self._need_final()
        if arr is None:
            arr = torch.zeros(self.num_cells, dtype=self.float_dtype, device=self.device)
        _lib.call("wcfd_div_flux", ct.byref(self.mesh_struct()), _ptr(self.mass_fluxes), _ptr(arr), _stream())
        return arr

    def replace_cell_values(self, output_indices, value):
        """cell_values[:, outs] = value laid out (C, n) row-major (model.py:318-325)."""
        idx = self._index_list(output_indices)
        assert len(idx) * self.num_cells == value.numel()
        v = value.reshape(self.num_cells, len(idx))
        for j, i in enumerate(idx):
            self.cell_values[:, i].copy_(v[:, j])

    def update_cell_values(self, field_idx, value, scale: float = 1.0):
        idx = self._index_list(field_idx)
        if isinstance(value, (float, int)):
            for i in idx:
                self.cell_values[:, i] += scale * float(value)
        else:
            v = value.reshape(self.num_cells, -1)
            for j, i in enumerate(idx):
                self.cell_values[:, i] += scale * v[:, min(j, v.shape[1] - 1)]

    def struct_member_to_array(self, member="centroid", struct="cells"):
        """Host copy of a per-cell or per-face geometric member (model.py:177-190)."""
        if struct == "cells":
            src = {"centroid": self.mesh._geometry64["centroid"], "volume": self.mesh._geometry64["volume"],
                   "faces": self.cell_properties.faces, "neighbors": self.cell_properties.neighbors}
        elif struct == "faces":
            src = {"centroid": self.mesh._geometry64["face_centroid"],
                   "adjacent_cells": self.face_properties.adjacent_cells,
                   "area": self._geo_host["face_normal"][:, 3] if self._geo is not None else None}
        else:
            raise ValueError("Only cell or face struct members can be returned")
        return np.asarray(src[member])

    def convergence_norms(self, vel_system, velocity, div_u=None, rua=None, p=None):
        """The nine residual norms of check_convergence from one fused device pass
        (wcfd_convergence_norms): ||A u - b||_2 and ||b||_2 per momentum component,
        ||div||_1, ||rUA grad p||_inf (from cell_gradients and rua), ||p||_inf."""
        if getattr(self, "_norm_scratch", None) is None:
            n = int(_lib.load().wcfd_convergence_scratch_floats())
            self._norm_scratch = torch.empty(n, dtype=torch.float32, device=self.device)
            self._norm_out = torch.empty(9, dtype=torch.float64, device=self.device)
        _lib.call("wcfd_convergence_norms", ct.byref(self.mesh_struct()), vel_system, _ptr(velocity),
                  _ptr(div_u) if div_u is not None else None,
                  _ptr(self.cell_gradients) if rua is not None else None,
                  _ptr(rua) if rua is not None else None, _ptr(p) if p is not None else None,
                  _ptr(self._norm_scratch), _ptr(self._norm_out), _stream())
        return self._norm_out.cpu().numpy()

    def check_convergence_norms(self, norms, log=True):
        """check_convergence from convergence_norms()."""
        conv = {}
        for o, name in enumerate(("momentum_x", "momentum_y", "momentum_z")):
            conv[name] = self.Convergence.check_norms(name, float(norms[o]), float(norms[3 + o]))
        conv["continuity"] = self.Convergence.check_norms("continuity", float(norms[6]))
        conv["local_continuity"] = self.Convergence.check_norms("local_continuity", float(norms[6]))
        conv["velocity_correction"] = self.Convergence.check_norms("velocity_correction", float(norms[7]))
        conv["pressure_correction"] = self.Convergence.check_norms("pressure_correction", float(norms[8]))
        if log:
            self.Convergence.log(conv)
        if np.isnan(conv["momentum_x"][0]):
            raise ValueError("NaN in the momentum residual")
        return conv, self.Convergence.has_converged()

    def check_convergence(self, vel_matrix, velocity, b, div_u=None, velocity_correction=None, p_correction=None,
                          log=True):
        """Residual norms of model.py:278-316 (fp64 on the device).  ``vel_matrix`` is a
        callable x -> A x (the solver passes its momentum SpMV)."""
        div_u = self.divFlux(div_u)
        Ax = vel_matrix(velocity).reshape(-1, 3).double()
        bb = b.reshape(-1, 3).double()
        conv = {}
        for o, name in enumerate(("momentum_x", "momentum_y", "momentum_z")):
            conv[name] = self.Convergence.check(name, Ax[:, o], bb[:, o])
        conv["continuity"] = self.Convergence.check("continuity", div_u.double())
        conv["local_continuity"] = self.Convergence.check("local_continuity", div_u.double().abs())
        conv["velocity_correction"] = (self.Convergence.check("velocity_correction", velocity_correction.double())
                                       if velocity_correction is not None else np.nan)
        conv["pressure_correction"] = (self.Convergence.check("pressure_correction", p_correction.double())
                                       if p_correction is not None else np.nan)
        if log:
            self.Convergence.log(conv)
        if np.isnan(conv["momentum_x"][0]):
            raise ValueError("NaN in the momentum residual")
        return conv, self.Convergence.has_converged()
