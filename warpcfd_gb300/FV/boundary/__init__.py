from .boundary import Boundary, DIRICHLET, NEUMANN
