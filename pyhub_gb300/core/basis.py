"""Many-body basis with the reference's API (pyhub/core/basis.py:8-261).

The reference enumerates spin strings with the Fortran program basis.x and
caches them in basis.h5 (basis.py:60-84, 167-171).  Here the strings come from
the C ABI (ed_basis, the same enumeration order as HILBERT,
compute_basis.f90:67-96) and are kept in memory; ``memspace`` is accepted for
signature compatibility and has no effect because there is no file cache.
"""
from __future__ import annotations

from itertools import product

import numpy as np

from .. import _capi


class Basis:

    def __init__(self, nb_sites: int, hilbert: tuple = None, order: str = "spin", memspace=None):
        self.nb_sites = nb_sites
        self.hilbert = hilbert
        if memspace is not None and not isinstance(memspace, str):
            raise ValueError(f"Set memspace as a correct string, not {memspace}")
        if isinstance(hilbert, tuple):
            if isinstance(hilbert[0], (int, np.integer)):
                self.nup = [int(hilbert[0])]
            elif isinstance(hilbert[0], (list, np.ndarray)):
                self.nup = [int(v) for v in hilbert[0]]
            else:
                raise ValueError(f"hilbert must be a tuple of n_up and n_down, not {hilbert}")
            if isinstance(hilbert[1], (int, np.integer)):
                self.ndown = [int(hilbert[1])]
            elif isinstance(hilbert[1], (list, np.ndarray)):
                self.ndown = [int(v) for v in hilbert[1]]
            else:
                raise ValueError(f"hilbert must be a tuple of n_up and n_down, not {hilbert}")
        elif hilbert is None:
            self.nup = np.array([i for i in range(self.nb_sites + 1)])
            self.ndown = np.array([i for i in range(self.nb_sites + 1)])
        else:
            raise ValueError(f"hilbert must be a tuple of n_up and n_down, not {hilbert}")
        if order != "site" and order != "spin":
            raise ValueError(f"basis order must be in site or spin convention, not {order}")
        try:
            self.order = order
        except AttributeError:  # subclasses may define order as a read-only property
            pass
        self._strings = {}

    def _strings_of(self, ne: int) -> np.ndarray:
        ne = int(ne)
        if ne not in self._strings:
            if ne < 0 or ne > self.nb_sites:
                self._strings[ne] = np.zeros(0, dtype=np.int64)
            else:
                self._strings[ne] = _capi.basis(self.nb_sites, ne).astype(np.int64)
        return self._strings[ne]

    def decompose(self, index):
        if self.order == "spin":
            return index & 2 ** self.nb_sites - 1, index >> self.nb_sites
        up, down = 0, 0
        for k in range(0, 2 * self.nb_sites, 2):
            if index & 2 ** k == 2 ** k:
                up += 2 ** (k // 2)
            if index & 2 ** (k + 1) == 2 ** (k + 1):
                down += 2 ** (k // 2)
        return up, down

    def __getitem__(self, index):
        if isinstance(index, np.ndarray):
            index = index.astype(int).tolist()
        if index == slice(None, None, None):
            return self.basis[:]
        return self.basis[index]

    def __iter__(self):
        return iter(self.basis)

    def __repr__(self):
        if self.order == "spin":
            return (f"basis up :\n{[up for up in self.basis_up]}\n"
                    f"basis down :\n{[down << self.nb_sites for down in self.basis_down]}")
        uplist = [self.site_ordering(int(up), 0)[0] for up in self.basis_up]
        downlist = [self.site_ordering(0, int(down))[1] for down in self.basis_down]
        return f"basis up :\n{uplist}\nbasis down :\n{downlist}"

    def bit_repr(self, index=None):
        if not isinstance(index, np.ndarray):
            index = np.array(range(self.nstates), dtype=int)
        string = "-" * (3 * (self.nb_sites + 4)) + "\n"
        string += "empty        : 0\nuparrow      : 1\ndownarrow    :-1\nupdoawnarrow : 2\n"
        string += "-" * (3 * (self.nb_sites + 4)) + "\n"
        string += "index | bit\n"
        string += "------|--" + "-" * (3 * (self.nb_sites + 1)) + "\n"
        for idx in self.basis[index]:
            up, down = self.decompose(int(idx))
            string += "{:4d}  |".format(int(idx))
            for i in range(self.nb_sites):
                u, d = (up >> i) & 1, (down >> i) & 1
                string += " 0 " if (not u and not d) else (" 1 " if (u and not d) else ("-1 " if (d and not u) else " 2 "))
            string += "\n"
        return string

    def spin_ordering(self, a, b):
        return a, (b << self.nb_sites)

    def site_ordering(self, a, b):
        a_new, b_new = 0, 0
        for i in range(self.nb_sites):
            a_new |= ((a >> i) & 1) << (2 * i)
            b_new |= ((b >> i) & 1) << (2 * i + 1)
        return a_new, b_new

    @property
    def filename_basis(self):
        return "basis.h5"

    def exec_basis(self, elem2comp):
        """The reference runs basis.x to enumerate the strings of the particle
        numbers elem2comp into basis.h5 (basis.py:167-171); here they are
        enumerated on demand by ed_basis, so this only warms the cache."""
        for ne in elem2comp:
            self._strings_of(int(ne))

    def __basisremove__(self):
        # the reference deletes basis.h5 (basis.py:85-89); no file is written here
        self._strings = {}

    @property
    def file_size(self):
        """Size of the reference's basis.h5; no file is written here."""
        return 0.0

    @property
    def basis(self):
        order = self.spin_ordering if self.order == "spin" else self.site_ordering
        return np.array([np.sum(order(int(up), int(down))) for down, up in product(self.basis_down, self.basis_up)],
                        dtype=int)

    @property
    def basis_up(self):
        return np.concatenate([self._strings_of(u) for u in self.nup])

    @property
    def basis_down(self):
        return np.concatenate([self._strings_of(d) for d in self.ndown])

    @property
    def nb_states(self):
        return self.nb_sup * self.nb_sdown

    @property
    def nb_sup(self):
        return int(np.sum([_capi.binom(self.nb_sites, int(u)) for u in self.nup]))

    @property
    def nb_sdown(self):
        return int(np.sum([_capi.binom(self.nb_sites, int(d)) for d in self.ndown]))

    @property
    def nstates(self):
        return self.nb_states

    @property
    def nsup(self):
        return self.nb_sup

    @property
    def nsdown(self):
        return self.nb_sdown

    @property
    def n_up(self):
        return self.nup

    @property
    def n_down(self):
        return self.ndown
