"""Hopping / exchange matrices of the clusters the engine is benchmarked on.

Amplitudes follow the reference's convention H = sum t_ij c^+_i c_j with
t_ij = -1 on nearest-neighbour bonds for "t = 1"
(examples/05-fermi_hubbard.py:11-13).  Sites are numbered s = x + lx*y.
"""
from __future__ import annotations

import numpy as np


def ring(n: int, t: float = -1.0) -> np.ndarray:
    m = np.zeros((n, n))
    for i in range(n):
        j = (i + 1) % n
        if j != i:
            m[i, j] = m[j, i] = t
    return m


def square(lx: int, ly: int, t: float = -1.0, periodic: bool = True, tp: float = 0.0) -> np.ndarray:
    """lx x ly square lattice; tp on the two diagonals of every plaquette."""
    n = lx * ly
    m = np.zeros((n, n))

    def link(a, b, v):
        if a != b:
            m[a, b] = m[b, a] = v

    for y in range(ly):
        for x in range(lx):
            s = x + lx * y
            for dx, dy in ((1, 0), (0, 1)):
                xx, yy = x + dx, y + dy
                if not periodic and (xx >= lx or yy >= ly):
                    continue
                link(s, (xx % lx) + lx * (yy % ly), t)
            if tp != 0.0:
                for dx, dy in ((1, 1), (1, -1)):
                    xx, yy = x + dx, y + dy
                    if not periodic and (xx >= lx or yy >= ly or yy < 0):
                        continue
                    link(s, (xx % lx) + lx * (yy % ly), tp)
    return m


def hubbard_4x4(U: float = 8.0):
    """4x4 periodic square lattice, t=1 (t_ij=-1), uniform U: the headline cluster."""
    return square(4, 4, -1.0, periodic=True), np.full(16, float(U))


def heisenberg_4x8(J: float = 1.0):
    """4x8 periodic square lattice (lx=4, ly=8), J_ij = J on the 64 bonds."""
    return square(4, 8, J, periodic=True)


def random_bond_cluster(n: int, n_extra: int, seed: int):
    """Ring of n sites plus n_extra distinct random non-ring bonds; t_ij ~ U[0.5,1.5]
    on all bonds, eps_i ~ N(0, 0.3^2) on the diagonal, U_i ~ U[2,6]."""
    rng = np.random.default_rng(seed)
    t = np.zeros((n, n))
    bonds = [(i, (i + 1) % n) for i in range(n)]
    ring_set = {tuple(sorted(b)) for b in bonds}
    cand = [(i, j) for i in range(n) for j in range(i + 1, n) if (i, j) not in ring_set]
    pick = rng.choice(len(cand), size=n_extra, replace=False)
    bonds += [cand[k] for k in sorted(pick)]
    for (i, j) in bonds:
        t[i, j] = t[j, i] = rng.uniform(0.5, 1.5)
    eps = rng.normal(0.0, 0.3, n)
    t[np.diag_indices(n)] = eps
    U = rng.uniform(2.0, 6.0, n)
    return t, U, [tuple(sorted(b)) for b in bonds]
