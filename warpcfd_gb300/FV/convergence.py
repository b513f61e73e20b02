"""Residual criteria and history (warp_cfd/FV/Convergence.py:7-99).

Norms are taken on the device in fp64; only the scalar results come to the host.
"""
from __future__ import annotations

import math

import torch


def _norm(x: torch.Tensor, ord):
    x = x.reshape(-1).double()
    if ord == math.inf or ord == float("inf"):
        return float(x.abs().max()) if x.numel() else 0.0
    if ord == 1:
        return float(x.abs().sum())
    if ord == 2:
        return float(torch.linalg.vector_norm(x))
    return float(x.abs().pow(ord).sum() ** (1.0 / ord))


class Criteria:
    def __init__(self, name, eps=1e-4, tol="relative", ord=1.0, is_flux=False) -> None:
        assert tol in ("relative", "abs")
        self.name = name
        self.eps = eps
        self.tol = tol
        self.ord = ord
        self.is_converged = False
        self.non_zero = 1e-6

    def residual(self, arr, rhs=0.0, ord=None):
        ord = self.ord if ord is None else ord
        return _norm(arr - rhs, ord)

    def relative_residual(self, arr, rhs, ord=None):
        ord = self.ord if ord is None else ord
        res = self.residual(arr, rhs, ord)
        rhs_norm = _norm(rhs, ord) if isinstance(rhs, torch.Tensor) else abs(float(rhs))
        return res / max(rhs_norm, self.non_zero)

    def check(self, arr, rhs=0.0, ord=None):
        if self.tol == "abs":
            res = self.residual(arr, rhs, ord)
        else:
            res = self.relative_residual(arr, rhs, ord)
        self.is_converged = res < self.eps
        return res, self.is_converged

    def check_norms(self, res_norm, rhs_norm=0.0):
        """check() from norms computed elsewhere (the device convergence monitor)."""
        res = res_norm if self.tol == "abs" else res_norm / max(rhs_norm, self.non_zero)
        self.is_converged = res < self.eps
        return res, self.is_converged


class Convergence:
    """Criteria of Convergence.py:53-61: continuity L1 abs 1e-4; momentum L2 relative
    1e-3; pressure/velocity corrections L-inf abs 1e-4."""

    def __init__(self):
        self.continuity = Criteria("continuity", eps=1e-4, tol="abs")
        self.local_continuity = Criteria("local_continuity", eps=1e-4, tol="abs")
        self.momentum_x = Criteria("momentum_x", ord=2.0, eps=1e-3)
        self.momentum_y = Criteria("momentum_y", ord=2.0, eps=1e-3)
        self.momentum_z = Criteria("momentum_z", ord=2.0, eps=1e-3)
        self.pressure_correction = Criteria("pressure_correction", tol="abs", eps=1e-4, ord=math.inf)
        self.velocity_correction = Criteria("velocity_correction", tol="abs", eps=1e-4, ord=math.inf)
        self.criterias = [self.continuity, self.momentum_x, self.momentum_y, self.momentum_z,
                          self.pressure_correction, self.velocity_correction]
        self.log_list = []

    def check(self, criteria: str, arr, rhs=0.0, ord=None):
        return getattr(self, criteria).check(arr, rhs, ord)

    def check_norms(self, criteria: str, res_norm, rhs_norm=0.0):
        return getattr(self, criteria).check_norms(res_norm, rhs_norm)

    def has_converged(self):
        return all(c.is_converged for c in self.criterias)

    def log(self, step: dict):
        self.log_list.append(step)
