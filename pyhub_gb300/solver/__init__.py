from .fermi_hubbard import FermiHubbard
from .heisenberg import Heisenberg

__all__ = ["FermiHubbard", "Heisenberg"]
