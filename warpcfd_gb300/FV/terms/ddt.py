"""DdtTerm (warp_cfd/FV/terms/ddt.py:7-32): backward Euler.  Calling the term with the time
step forms its (C, n, 2) weights (V/dt, -phi V/dt) on the device (wcfd_ddt_weights)."""
import ctypes as ct

import torch

from ... import _lib
from .terms import Term


class DdtTerm(Term):
    def __init__(self, fv, fields, time_scheme="backwardEuler") -> None:
        super().__init__(fv, fields, implicit=True, need_global_index=True, cell_based=True)
        if time_scheme != "backwardEuler":
            raise NotImplementedError("Only backwardEuler valid option now")
        self.time_scheme = time_scheme
        self.dt = None

    def calculate_weights(self, fv, dt=None, **kwargs):
        if dt is not None:
            self.dt = float(dt)
        if self.dt is None:
            raise ValueError("call the ddt term with its time step: ddt(model, dt=dt)")
        w = self._weights_for(fv)
        _lib.call("wcfd_ddt_weights", ct.byref(fv.mesh_struct()), fv.state_struct(), self.field_struct(),
                  float(self.dt), ct.c_void_p(w.data_ptr()), ct.c_void_p(torch.cuda.current_stream().cuda_stream))
        return self
