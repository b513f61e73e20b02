"""DdtTerm (warp_cfd/FV/terms/ddt.py:7-32): backward Euler V/dt on the diagonal and
phi_old V/dt on the RHS, formed in the momentum assembly kernel when steady_state=False."""
from .terms import Term


class DdtTerm(Term):
    def __init__(self, fv, fields, time_scheme="backwardEuler") -> None:
        super().__init__(fv, fields, implicit=True, need_global_index=True, cell_based=True)
        if time_scheme != "backwardEuler":
            raise NotImplementedError("Only backwardEuler valid option now")
        self.time_scheme = time_scheme
        self.dt = None

    def calculate_weights(self, fv, dt=None, **kwargs):
        """Records the time step of the next form_system (ddt.py:24-32)."""
        if dt is not None:
            self.dt = float(dt)
        return self
