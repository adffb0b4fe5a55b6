"""Elementary operators with the reference's API (pyhub/tools/operators.py:1-159).

Each class is a one-term Operators whose string names the elementary
operator; sums and products build general operators (core/_operators.py).
Sites are 0-based; spins 'u'/'up'/1/'+' are up, anything else down.
"""
from __future__ import annotations

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
