"""Term algebra (warp_cfd/FV/terms/terms.py:8-113).

A term names the fields it acts on and carries a scale.  As in the reference the scale
is ASSIGNED, not multiplied: ``-t`` sets it to -1 and ``c * t`` sets it to c
(terms.py:88-113), so ``-inv_density * grad_P`` has scale -1/rho.

Calling a term (``term(model, ...)``) forms its weights on the device in the reference's
layouts (libwcfd ``wcfd_*_weights``): face-based implicit terms (C, F, n, 3) = (owner,
neighbour, explicit) per cell side of each face, cell-based implicit terms (C, n, 2) =
(diagonal, explicit), explicit terms (3C,).  ``Equation.form_system`` adds any list of them
into its system.  The weights array is allocated on the first call (shared by the shallow
copies ``-t`` and ``c * t`` make, as in the reference).
"""
from __future__ import annotations

import copy
import ctypes

import torch

from ..field import Field


class Term:
    def __init__(self, fv, fields, implicit, need_global_index: bool, cell_based: bool) -> None:
        self.fields = []
        if need_global_index:
            if isinstance(fields, str):
                fields = [fields]
            for name in fields:
                if name not in fv.output_variables:
                    raise ValueError(f"Field {name} was not found in original model only variables "
                                     f"{fv.output_variables} are available")
                self.fields.append(fv.fields[name])
        else:
            assert isinstance(fields, str), "Only one field variable can be defined if global index is False"
            self.fields.append(Field(fields, index=-1))
        self.global_output_indices = [f.index for f in self.fields]
        self.need_global_index = need_global_index
        self.local_field_index = {f.name: i for i, f in enumerate(self.fields)}
        self.num_outputs = len(self.fields)
        self._implicit = implicit
        self.cell_based = cell_based
        self.float_dtype = fv.float_dtype
        self._scale = 1.0
        self._holder = {"weights": None}   # shared with the shallow copies of -t and c * t

    @property
    def weights(self):
        """The device weights of the last call (None before the first)."""
        return self._holder["weights"]

    def _weights_for(self, fv):
        """The weights array in this term's layout, allocated on first use."""
        w = self._holder["weights"]
        if w is None:
            C, F, n = fv.num_cells, fv.faces_per_cell, self.num_outputs
            shape = (C, n, 2) if self.cell_based else ((C, F, n, 3) if self.implicit else (3 * C,))
            w = torch.zeros(shape, dtype=torch.float32, device=fv.device)
            self._holder["weights"] = w
        return w

    def field_struct(self):
        """The C struct of the term's fields.  A term built with need_global_index=False
        reads column 0, as the reference's does (its global index array is zeros(1),
        terms.py:37-39)."""
        from ... import _lib

        idx = [max(i, 0) for i in self.global_output_indices] if self.need_global_index else [0]
        return _lib.TermFields_t(len(idx), (ctypes.c_int32 * 3)(*(idx + [0] * (3 - len(idx)))))

    def set_implicit(self, implicit: bool):
        self._implicit = implicit

    def set_scale(self, value):
        self._scale = float(value)

    @property
    def scale(self):
        return self._scale

    @property
    def implicit(self):
        return self._implicit

    def __pos__(self):
        self.set_scale(1.0)
        return self

    def __neg__(self):
        t = copy.copy(self)
        t.set_scale(-1.0)
        return t

    def __call__(self, fv, *args, **kwargs):
        return self.calculate_weights(fv, *args, **kwargs)

    def calculate_weights(self, fv, *args, **kwargs):
        pass

    def __mul__(self, value):
        if isinstance(value, (float, int)):
            t = copy.copy(self)
            t.set_scale(value)
            return t
        return NotImplemented

    def __rmul__(self, other):
        return self.__mul__(other)
