"""ORACLE test infrastructure: warp.optim of the numpy Warp stand-in."""
from . import linear  # noqa: F401
