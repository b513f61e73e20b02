"""ConvectionTerm (warp_cfd/FV/terms/convection.py:8-91).

Calling the term forms its (C, F, n, 3) weights on the device (wcfd_convection_weights):
upwind, central difference or upwindLinear (Implicit_Schemes/convectionScheme.py:3-88),
with the skew correction in the explicit part as the reference's term always applies it.
The incompressible solver's fused momentum assembly forms the same coefficients inside
its own kernel and does not call the term."""
import ctypes as ct

import torch

from ... import _lib
from .terms import Term

SCHEMES = ("upwind", "central difference", "upwindLinear", "custom")
_CODES = {"upwind": 0, "central difference": 1, "upwindLinear": 2}


class ConvectionTerm(Term):
    def __init__(self, fv, fields, interpolation="upwind", custom_interpolation=None):
        super().__init__(fv, fields, implicit=True, need_global_index=True, cell_based=False)
        assert interpolation in SCHEMES, "interpolation schems supported: upwind, central difference, " \
                                         "upwindLinear or custom"
        if interpolation == "custom":
            assert custom_interpolation is not None
        self.interpolation = interpolation
        self.custom_interpolation = custom_interpolation
        self.correct_face_interpolation = True

    def calculate_weights(self, fv, **kwargs):
        if self.interpolation == "custom":
            raise NotImplementedError("a custom interpolation is a Warp function in the reference; this path "
                                      "forms upwind, central difference and upwindLinear weights")
        w = self._weights_for(fv)
        _lib.call("wcfd_convection_weights", ct.byref(fv.mesh_struct()), fv.state_struct(), self.field_struct(),
                  _CODES[self.interpolation], ct.c_void_p(w.data_ptr()),
                  ct.c_void_p(torch.cuda.current_stream().cuda_stream))
        return self
