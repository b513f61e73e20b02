"""DiffusionTerm (warp_cfd/FV/terms/diffusion.py:8-198): configuration holder; the
coefficients nu A/|d| (x |n1| with correction) are formed in the assembly kernels."""
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
        self.correction = correction
        self.von_neumann = von_neumann
        self.dirchlet = dirchlet
        self.viscosity = None

    def calculate_weights(self, fv, viscosity=None, **kwargs):
        """Records the viscosity of the next form_system: a scalar, or a tensor of one value
        per face (diffusion.py:113-198 forms the weights here; the assembly kernels do)."""
        if viscosity is not None:
            self.viscosity = viscosity
        return self
