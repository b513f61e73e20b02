from .model import FVM
