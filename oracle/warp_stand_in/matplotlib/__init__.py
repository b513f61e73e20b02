"""ORACLE test infrastructure: a stand-in for matplotlib, which warp_cfd's
FV/Convergence.py imports at module level for plotting only."""
