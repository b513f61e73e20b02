from .incompressible import IncompressibleSolver
from .solverSchemes import SIMPLE, PISO
