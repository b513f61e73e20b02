from .mesh import Mesh, UnstructuredGrid, HEXAHEDRON, WEDGE, TETRA
from .grid import (create_2D_grid, create_3D_grid, create_cylinder_channel_grid, define_boundary_walls,
                   define_cylinder_group, jitter_interior_nodes)

__all__ = ["Mesh", "UnstructuredGrid", "define_boundary_walls", "create_2D_grid", "create_3D_grid",
           "jitter_interior_nodes", "create_cylinder_channel_grid", "define_cylinder_group", "HEXAHEDRON", "WEDGE", "TETRA"]
