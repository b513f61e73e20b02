"""ConvectionTerm (warp_cfd/FV/terms/convection.py:8-91).

In the incompressible solver the upwind convection coefficients are formed inside the
fused momentum assembly kernel; this class carries the term's configuration."""
from .terms import Term

SCHEMES = ("upwind", "central difference", "upwindLinear", "custom")


class ConvectionTerm(Term):
    def __init__(self, fv, fields, interpolation="upwind", custom_interpolation=None):
        super().__init__(fv, fields, implicit=True, need_global_index=True, cell_based=False)
        assert interpolation in SCHEMES, "interpolation schems supported: upwind, central difference, " \
                                         "upwindLinear or custom"
        if interpolation == "custom":
            assert custom_interpolation is not None
        self.interpolation = interpolation
        self.correct_face_interpolation = True
