from .mat import Material
