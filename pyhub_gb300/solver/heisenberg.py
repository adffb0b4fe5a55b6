"""Heisenberg with the reference's signature (pyhub/solver/heisenberg.py:13-66):
the Sz=0 sector stored as (n_up=N/2, n_down=0) strings, the down string being
the complement of the up string."""
import numpy as np

from ..core.core_solver import CoreSolver


class Heisenberg(CoreSolver):
    r"""
    Sz=0 Heisenberg model  H = \sum_{JK} J_{JK} S_J . S_K  (ordered pairs, as
    the reference sums them), solved on the GPU.
    """

    def __init__(self, nb_sites, J_matrix: np.ndarray, T=0.):
        CoreSolver.__init__(self, nb_sites, nb_sites // 2, 0, 'heisenberg.x', T)
        self.J_matrix = J_matrix
        if not np.isclose(self.J_matrix, self.J_matrix.T).all():
            raise ValueError('J_matrix must be symmetric')

    @property
    def filename(self):
        return 'solver.h5'

    def __fileremove__(self):
        pass

    @property
    def order(self):
        return 'spin'

    def bit_repr(self, index=None):
        if not isinstance(index, np.ndarray):
            index = np.array(range(self.nstates), dtype=int)
        string = '-' * (3 * (self.nb_sites + 4)) + '\n'
        string += 'empty        : 0\nuparrow      : 1\ndownarrow    :-1\nupdoawnarrow : 2\n'
        string += '-' * (3 * (self.nb_sites + 4)) + '\n'
        string += 'index | bit\n'
        string += '------|--' + '-' * (3 * (self.nb_sites + 1)) + '\n'
        for idx in self.basis[index]:
            up = int(idx) & 2 ** self.nb_sites - 1
            down = 2 ** self.nb_sites - 1 - up
            string += "{:4d}  |".format(int(idx))
            for i in range(self.nb_sites):
                u, d = (up >> i) & 1, (down >> i) & 1
                string += ' 0 ' if (not u and not d) else (' 1 ' if (u and not d) else ('-1 ' if (d and not u) else ' 2 '))
            string += '\n'
        return string
