"""Solver helper kernels of the reference's run loop (warp_cfd/FV/kernels/solver_kernels.py)."""
from .solver_kernels import calculate_rUA, get_HbyA, interpolate_cell_value_to_face

__all__ = ["calculate_rUA", "get_HbyA", "interpolate_cell_value_to_face"]
