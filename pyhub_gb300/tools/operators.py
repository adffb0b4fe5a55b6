"""Elementary operators with the reference's API (pyhub/tools/operators.py:1-159).

Each class is a one-term Operators whose string names the elementary
operator; sums and products build general operators (core/_operators.py).
Sites are 0-based; spins 'u'/'up'/1/'+' are up, anything else down.
"""
from __future__ import annotations

import numpy as np

from ..core._operators import Operators


class c_dagger_c(Operators):
    def __init__(self, *args):
        Operators.__init__(self, *args)
        self.str_index = [["c_dagger_c"]]


class c_dagger(Operators):
    def __init__(self, *args):
        Operators.__init__(self, *args)
        self.str_index = [["c_dagger"]]


class _c(Operators):
    def __init__(self, *args):
        Operators.__init__(self, *args)
        self.str_index = [["c"]]


class n(Operators):
    def __init__(self, *args):
        Operators.__init__(self, *args)
        self.str_index = [["n"]]


class _n(Operators):
    """1 - n."""
    def __init__(self, *args):
        Operators.__init__(self, *args)
        self.str_index = [["1_n"]]


class sz(Operators):
    def __init__(self, *args):
        Operators.__init__(self, *args)
        self.str_index = [["sz"]]


class splus(Operators):
    def __init__(self, *args):
        Operators.__init__(self, *args)
        self.str_index = [["splus"]]


class sminus(Operators):
    def __init__(self, *args):
        Operators.__init__(self, *args)
        self.str_index = [["sminus"]]


class idt(Operators):
    def __init__(self):
        Operators.__init__(self)
        self.coeff = [1.0]
        self.elem_index = [[()]]
        self.str_index = [["id."]]


class empty_operator(Operators):
    def __init__(self):
        Operators.__init__(self)
        self.coeff = []
        self.elem_index = []
        self.str_index = []


def sisj(*args):
    """S_i.S_j as the reference builds it (pyhub/tools/operators.py:41-51):
    i != j: -(c^+_iu c_ju c^+_jd c_id + c^+_id c_jd c^+_ju c_iu)/2 + sz_i sz_j;
    i == j: n_iu (1 - n_id)/2 taken twice, + sz_i sz_i."""
    op = empty_operator()
    i, j = args[0][0], args[1][0]
    if i == j:
        op += n((i, "up")) * _n((i, "down")) / 2 + n((i, "up")) * _n((i, "down")) / 2
    else:
        op -= (c_dagger_c((i, "u"), (j, "u")) * c_dagger_c((j, "d"), (i, "d"))
               + c_dagger_c((i, "d"), (j, "d")) * c_dagger_c((j, "u"), (i, "u"))) / 2
    op += sz((i,)) * sz((j,))
    return op


def opesum(lst):
    H = empty_operator()
    for op in lst:
        H += op
    return H


def opeexp(op, psi, ftol=1.e-6, unitary=False):
    """exp(op) psi by its Taylor series (pyhub/tools/operators.py:91-111): terms
    op^k psi / k! added until the squared norm of the sum changes by less than
    ftol between terms (unitary: differs from ||psi|| by less than ftol),
    at most 99 terms; the products op @ v run on the GPU."""
    if isinstance(psi, (list, np.ndarray)):
        psi = np.asarray(psi)
        conv = False
        new_psi, full_psi, i, val = np.copy(psi), np.copy(psi), 1, 1.e3
        nmr0 = np.linalg.norm(psi)
        while not conv and i < 100:
            new_psi = op @ new_psi / i
            full_psi += new_psi
            i += 1
            nmr = full_psi.conj() @ full_psi
            if unitary:
                if np.abs(nmr0 - nmr) < ftol:
                    conv = True
            else:
                if np.abs(val - nmr) < ftol:
                    conv = True
                else:
                    val = nmr
        if i == 100:
            raise ValueError('exponential operator does not converge')
        return full_psi
    # no vector: the matrix whose row i is exp(op) applied to basis state i
    matrix = np.zeros((op.nb_selected, op.nb_selected))
    psi0 = np.zeros(op.nb_selected)
    for i in range(op.nb_selected):
        psi0[i] = 1.
        matrix[i, :] = opeexp(op, psi0)
        psi0[i] = 0.
    return matrix

