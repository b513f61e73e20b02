"""The helpers IncompressibleSolver.run calls between its solves
(warp_cfd/FV/kernels/solver_kernels.py:6-43), for loops written against the reference's
API.  Each is one kernel of libwcfd.so on the current stream; the fused step computes the
same values with the same expressions.  Where the reference passes its cell or face struct
arrays, these take the model."""
from __future__ import annotations

import ctypes as ct

import torch

from ... import _lib


def _stream():
    return ct.c_void_p(torch.cuda.current_stream().cuda_stream)


def calculate_rUA(Ap, density, model, rUA=None):
    """rUA = V / (a_P rho), a_P the u-row diagonal of the momentum system
    (solver_kernels.py:6-16)."""
    if rUA is None:
        rUA = torch.empty(model.num_cells, dtype=torch.float32, device=model.device)
    _lib.call("wcfd_rua", ct.byref(model.mesh_struct()), ct.c_void_p(Ap.data_ptr()), float(density),
              ct.c_void_p(rUA.data_ptr()), _stream())
    return rUA


def get_HbyA(HbyA, rUA, p_grad):
    """HbyA += rUA grad p on 3C interleaved rows (solver_kernels.py:38-43); returns HbyA."""
    n = rUA.numel()
    assert HbyA.numel() == 3 * n and p_grad.numel() == 3 * n
    _lib.call("wcfd_hbya_add", int(n), ct.c_void_p(p_grad.contiguous().data_ptr()), ct.c_void_p(rUA.data_ptr()),
              ct.c_void_p(HbyA.data_ptr()), _stream())
    return HbyA


def interpolate_cell_value_to_face(face_array, cell_array, model):
    """Linear (psi-weighted) cell-to-face interpolation, the owner's value on boundary
    faces (solver_kernels.py:21-36); returns face_array."""
    if face_array is None:
        face_array = torch.empty(model.num_faces, dtype=torch.float32, device=model.device)
    _lib.call("wcfd_cell_to_face", ct.byref(model.mesh_struct()), ct.c_void_p(cell_array.data_ptr()),
              ct.c_void_p(face_array.data_ptr()), _stream())
    return face_array
