"""Term algebra (warp_cfd/FV/terms/terms.py:8-113).

A term names the fields it acts on and carries a scale.  As in the reference the scale
is ASSIGNED, not multiplied: ``-t`` sets it to -1 and ``c * t`` sets it to c
(terms.py:88-113), so ``-inv_density * grad_P`` has scale -1/rho.
"""
from __future__ import annotations

import copy

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
        self.weights = None

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
