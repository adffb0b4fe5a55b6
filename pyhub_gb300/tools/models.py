"""Model operators with the reference's API (pyhub/tools/models.py:5-14)."""
from __future__ import annotations

from itertools import product

import numpy as np

from .operators import c_dagger_c, n, opesum, sisj


def fermi_hubbard(t_matrix, U):
    """sum_{i,j,s} t[i,j] c^+_{i s} c_{j s} + sum_i U_i n_{i up} n_{i down}."""
    nb_sites = t_matrix.shape[0]
    if isinstance(U, (float, int)):
        U = np.full(nb_sites, U)
    return (opesum([t_matrix[i, j] * c_dagger_c((i, spin), (j, spin))
                    for i, j, spin in product(range(nb_sites), range(nb_sites), ["up", "down"])])
            + opesum([U[i] * n((i, "up")) * n((i, "down")) for i in range(nb_sites)]))


def heisenberg(J_matrix):
    """sum_{i,j} J[i,j] sisj(i,j) on the fermionic (N_up, N_down) basis."""
    nb_sites = J_matrix.shape[0]
    return opesum([J_matrix[i, j] * sisj((i,), (j,)) for i, j in product(range(nb_sites), range(nb_sites))])
