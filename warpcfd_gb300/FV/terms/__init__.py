from .convection import ConvectionTerm
from .diffusion import DiffusionTerm
from .grad import GradTerm
from .equation import Equation
from .ddt import DdtTerm
from .terms import Term
