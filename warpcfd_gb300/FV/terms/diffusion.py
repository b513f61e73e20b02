"""DiffusionTerm (warp_cfd/FV/terms/diffusion.py:8-198).

Calling the term with its viscosity forms its (C, F, n, 3) weights on the device
(wcfd_diffusion_weights): nu A (-1/|d|, 1/|d|) on internal faces, with |n1| and the
explicit non-orthogonal part when ``correction`` (laplacianScheme.py:14-67), and the
boundary weights from the boundary table (or a uniform normal gradient with the
``von_neumann`` / ``dirchlet`` options, both of which the reference builds with its von
Neumann kernel, diffusion.py:26-35).  The viscosity is a float or a device tensor of one
value per face (or a single value)."""
import ctypes as ct

import torch

from ... import _lib
from .terms import Term


class DiffusionTerm(Term):
    def __init__(self, fv, fields, *, correction=False, custom_interpolation=None, von_neumann=None, dirchlet=None,
                 need_global_index=True):
        super().__init__(fv, fields, implicit=True, need_global_index=need_global_index, cell_based=False)
        if correction:
            assert need_global_index, "Fields Must be defined in the FVM model to use corrections"
        assert custom_interpolation is None, "Custom laplacian functions not available yet"
        assert not ((von_neumann is not None) and (dirchlet is not None)), \
            "von neumann and dirichlet settings cannot both be not None"
        if von_neumann is not None or dirchlet is not None:
            assert len(self.fields) == 1, "Von neumann or dirichlet option only valid if len of field == 1"
        self.correction = correction
        self.von_neumann = von_neumann
        self.dirchlet = dirchlet
        self.viscosity = None

    def calculate_weights(self, fv, viscosity=None, **kwargs):
        if viscosity is not None:
            self.viscosity = viscosity
        nu = self.viscosity
        if nu is None:
            raise ValueError("call the diffusion term with its viscosity: diffusion(model, viscosity=nu)")
        nu_faces = None
        if torch.is_tensor(nu):
            if nu.numel() == 1:
                nu = float(nu.reshape(-1)[0].item())
            elif nu.numel() == fv.num_faces:
                nu_faces = nu.to(device=fv.device, dtype=torch.float32).contiguous()
                self._nu_faces = nu_faces          # keeps the buffer alive for the launch
                nu = 0.0
            else:
                raise ValueError("a viscosity tensor has one value per face or a single value")
        uniform = self.von_neumann if self.von_neumann is not None else self.dirchlet
        w = self._weights_for(fv)
        _lib.call("wcfd_diffusion_weights", ct.byref(fv.mesh_struct()), fv.bc_struct(), fv.state_struct(),
                  self.field_struct(), float(nu), ct.c_void_p(nu_faces.data_ptr() if nu_faces is not None else 0),
                  int(bool(self.correction)), 0 if uniform is None else 1, float(uniform or 0.0),
                  ct.c_void_p(w.data_ptr()), ct.c_void_p(torch.cuda.current_stream().cuda_stream))
        return self
