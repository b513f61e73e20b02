"""GradTerm (warp_cfd/FV/terms/grad.py:7-29): explicit grad(field) V source."""
from .terms import Term


class GradTerm(Term):
    def __init__(self, fv, field: str) -> None:
        assert isinstance(field, str), "grad Term can only be in terms of 1 field string name only"
        super().__init__(fv, field, implicit=False, need_global_index=True, cell_based=False)
