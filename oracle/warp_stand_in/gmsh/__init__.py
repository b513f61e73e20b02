"""ORACLE test infrastructure: an empty stand-in for gmsh, which warp_cfd's
preprocess/grid.py imports at module level; the reference fixtures build their meshes
without it."""
