"""GradTerm (warp_cfd/FV/terms/grad.py:7-29): the explicit source grad(field) V.  Calling the
term forms its (3C,) weights on the device (wcfd_grad_weights), rows 3c + d."""
import ctypes as ct

import torch

from ... import _lib
from .terms import Term


class GradTerm(Term):
    def __init__(self, fv, field: str) -> None:
        assert isinstance(field, str), "grad Term can only be in terms of 1 field string name only"
        super().__init__(fv, field, implicit=False, need_global_index=True, cell_based=False)

    def calculate_weights(self, fv, **kwargs):
        w = self._weights_for(fv)
        _lib.call("wcfd_grad_weights", ct.byref(fv.mesh_struct()), fv.state_struct(), int(self.fields[0].index),
                  ct.c_void_p(w.data_ptr()), ct.c_void_p(torch.cuda.current_stream().cuda_stream))
        return self
