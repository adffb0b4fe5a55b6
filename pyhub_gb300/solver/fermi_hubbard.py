"""FermiHubbard with the reference's signature (pyhub/solver/fermi_hubbard.py:13-29)."""
import numpy as np

from ..core.core_solver import CoreSolver


class FermiHubbard(CoreSolver):
    r"""
    General Hubbard cluster solved by exact diagonalisation or Lanczos on the
    GPU:  H = \sum_{ij\sigma} t_{ij} c^\dagger_{i\sigma} c_{j\sigma} + \sum_i U_i n_{i\uparrow} n_{i\downarrow}
    """

    def __init__(self, nb_sites, n_up: int, n_down: int, t_matrix: np.ndarray, U: float = 0, T=0., order='spin'):
        CoreSolver.__init__(self, nb_sites, n_up, n_down, 'hubbard.x', T, order=order)
        self.t_matrix = t_matrix
        if not np.isclose(self.t_matrix, self.t_matrix.T).all():
            raise ValueError('t_matrix must be symmetric')
        self.ek, self.Vk = np.linalg.eigh(self.t_matrix)
        self.U = U

    def __fileremove__(self):
        pass
