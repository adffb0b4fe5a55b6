"""Operator algebra with the reference's API (pyhub/core/_operators.py:10-365),
evaluated on the GPU when the operator has Hubbard form.

The reference keeps an operator as a sum of products of elementary
operators (c_dagger_c, n, 1_n, sz, id., ...) and applies it to a vector by
writing the term list and the vector to operators.h5 and running the Fortran
program operators.x once per product (`__call__`, :148-205; `to_matrix`,
:254-281; `lanczos`, :283-322).  Here the same term list is kept in memory
and recognised:

* Hubbard form -- sums of c^+_{i s} c_{j s} (both spins with the same
  coefficient matrix), n_{i s} and n_{i up} n_{i down} terms and the
  identity -- is a sector of the engine: ``@``, ``avg``, ``to_matrix`` and
  ``lanczos`` run the GPU H*v of a sector built from the recognised
  (t, U).  operators.x applies c^+_J c_K with the same KINOP/ANTICOM signs
  and the same (d-1)*NSUP+u index as HPROD (operators.f90:1-60), so the
  results are the reference's.
* One-body terms of either spin, densities, n_{i up} n_{i down} and the
  spin correlation sisj((i,),(j,)) built by pyhub.tools.operators.sisj are
  evaluated by ``avg`` through the fused RDM kernel (ed_rdm).

Other products (c_dagger, c, splus, sminus, operators mixing sectors) need
the generic engine, which is not built: they raise NotImplementedError, as
does a basis that holds more than one (N_up, N_down) sector or a selection
of states.
"""
from __future__ import annotations

import re
from itertools import product

import numpy as np

from .basis import Basis
from .. import _capi


def _torch():
    import torch
    return torch


def _is_up(spin) -> bool:
    return spin == 1 or spin == "u" or spin == "up" or spin == "+"


class Operators(Basis):

    def __init__(self, *args):
        self.coeff = [1.0]
        self.elem_index = [[(args)]]
        self.op2write = True

    # ------------------------------------------------------------ algebra
    def __add__(self, other):
        add = Operators.empty_operator()
        if isinstance(other, Operators):
            add.coeff = self.coeff + other.coeff
            add.elem_index = self.elem_index + other.elem_index
            add.str_index = self.str_index + other.str_index
        elif isinstance(other, (float, int)):
            return self + other * Operators._idt()
        return add

    def __radd__(self, other):
        return self.__add__(other)

    def __sub__(self, other):
        sub = Operators.empty_operator()
        if isinstance(other, Operators):
            sub.coeff = self.coeff + [-1.0 * c for c in other.coeff]
            sub.elem_index = self.elem_index + other.elem_index
            sub.str_index = self.str_index + other.str_index
        elif isinstance(other, (float, int)):
            return self - other * Operators._idt()
        return sub

    def __rsub__(self, other):
        return -1 * self.__sub__(other)

    def __mul__(self, other):
        mul = Operators.empty_operator()
        if isinstance(other, Operators):
            mul.coeff = [c1 * c2 for c1, c2 in product(self.coeff, other.coeff)]
            mul.elem_index = [[*c1, *c2] for c1, c2 in product(self.elem_index, other.elem_index)]
            mul.str_index = [[*c1, *c2] for c1, c2 in product(self.str_index, other.str_index)]
        elif isinstance(other, (float, int)):
            mul.coeff = [other * c for c in self.coeff]
            mul.elem_index = self.elem_index
            mul.str_index = self.str_index
            if not self.op2write:
                mul.set_basis(Basis(self.nb_sites, self.hilbert, self.order))
        return mul

    def __rmul__(self, other):
        return self.__mul__(other)

    def __neg__(self):
        return self.__mul__(-1.0)

    def __truediv__(self, other):
        if isinstance(other, (float, int)):
            return self.__mul__(1 / float(other))
        return NotImplemented

    def __matmul__(self, other):
        return self.__call__(other)

    def __rmatmul__(self, other):
        return self.__call__(other.conj())

    @staticmethod
    def empty_operator():
        empty = Operators()
        empty.coeff = []
        empty.elem_index = []
        empty.str_index = []
        return empty

    @staticmethod
    def _idt():
        idt = Operators()
        idt.coeff = [1.0]
        idt.elem_index = [[()]]
        idt.str_index = [["id."]]
        return idt

    @property
    def nb_ope(self):
        return len(self.coeff)

    def __repr__(self):
        return self.__str__()

    def __str__(self):
        full = ""
        for i, coeff in enumerate(self.coeff):
            s = f"{np.around(coeff, 3)}*"
            for j, elem in enumerate(self.elem_index[i]):
                s += _print_from_string(self.str_index[i][j], elem)
            full += s + " + "
        full = re.sub(r"\*\s", r" ", full)
        full = re.sub(r"(.*) \+ $", r"\1", full)
        return re.sub(r"\+\s-", r"- ", full)

    # ------------------------------------------------------------ basis
    def set_basis(self, B: Basis, selected: np.ndarray = None, memspace="10Go"):
        Basis.__init__(self, B.nb_sites, hilbert=B.hilbert, order=B.order)
        self.nb_selected = len(selected) if isinstance(selected, np.ndarray) else self.nstates
        self.selected = selected if isinstance(selected, np.ndarray) else None
        self.op2write = False
        self._sector = None
        self._lcz = None

    def _check_basis(self):
        if self.op2write:
            raise AttributeError("Set the basis set using self.set_basis(YourBasis:Basis)")
        if self.selected is not None:
            raise NotImplementedError("operators on a selection of basis states need the generic operator engine")
        if len(self.n_up) != 1 or len(self.n_down) != 1:
            raise NotImplementedError("operators on a basis of several (N_up, N_down) sectors need the generic "
                                      "operator engine")

    # ------------------------------------------------------------ recognition
    def _classify(self):
        """(t_up, t_down, U, const, rest): the one-body coefficient matrices of
        each spin (element [i][j] multiplies c^+_i c_j), the local U, the
        identity coefficient, and the terms that are not of that form."""
        N = self.nb_sites
        tu, td, U = np.zeros((N, N)), np.zeros((N, N)), np.zeros(N)
        const = 0.0
        rest = []
        for c, strs, elems in zip(self.coeff, self.str_index, self.elem_index):
            if strs == ["id."]:
                const += c
            elif strs == ["c_dagger_c"] and _is_up(elems[0][0][1]) == _is_up(elems[0][1][1]):
                (i, s), (j, _) = elems[0]
                (tu if _is_up(s) else td)[i, j] += c
            elif strs == ["n"]:
                i, s = elems[0][0]
                (tu if _is_up(s) else td)[i, i] += c
            elif strs == ["n", "n"] and elems[0][0][0] == elems[1][0][0] and \
                    _is_up(elems[0][0][1]) != _is_up(elems[1][0][1]):
                U[elems[0][0][0]] += c
            else:
                rest.append((c, strs, elems))
        return tu, td, U, const, rest

    def _hubbard(self):
        """(t, U, const) when the operator has Hubbard form, else None."""
        tu, td, U, const, rest = self._classify()
        if rest or np.abs(tu - td).max(initial=0.0) > 0.0:
            return None
        return tu, U, const

    def _sector_of(self):
        if self._sector is None:
            h = self._hubbard()
            if h is None:
                raise NotImplementedError("applying this operator needs the generic operator engine: only the Hubbard "
                                          "form (same hopping for both spins, n, n_up n_down, identity) runs on the "
                                          "GPU sector product")
            t, U, const = h
            sec = _capi.Sector(self.nb_sites, int(self.n_up[0]), int(self.n_down[0]), _capi.ED_HUBBARD, t=t, U=U)
            self._sector = (sec, const)
        return self._sector

    # ------------------------------------------------------------ application
    def _apply(self, psi: np.ndarray) -> np.ndarray:
        torch = _torch()
        sec, const = self._sector_of()
        x = sec.from_ref(torch.tensor(np.asarray(psi, dtype=np.float64), device="cuda"))
        y = torch.zeros_like(x)
        sec.hv(x, y)
        if const != 0.0:
            y.add_(x, alpha=const)
        return sec.to_ref(y).cpu().numpy()

    def __call__(self, psi, avg=False):
        self._check_basis()
        psi = np.asarray(psi)
        if np.iscomplexobj(psi):
            if not avg:
                return self.__call__(psi.real, avg=False) + 1j * self.__call__(psi.imag, avg=False)
            return self.__call__(psi.real, avg=True) + self.__call__(psi.imag, avg=True)
        if avg:
            return self._expectation(psi)
        return self._apply(psi)

    def avg(self, psi):
        return self.__call__(psi, avg=True)

    def _expectation(self, psi: np.ndarray) -> float:
        if self._hubbard() is not None:
            return float(psi @ self._apply(psi))
        return self._rdm_expectation(psi)

    def _rdm_expectation(self, psi: np.ndarray) -> float:
        """<psi|O|psi> from the fused RDM pass, for one-body terms of either
        spin, densities, n_up n_down and the spin correlations of sisj."""
        torch = _torch()
        N = self.nb_sites
        tu, td, U, const, rest = self._classify()
        # sisj((i,),(j,)), i != j (pyhub/tools/operators.py:41-51): -1/2 (c^+_iu c_ju c^+_jd c_id +
        # c^+_id c_jd c^+_ju c_iu) + sz_i sz_j; the two exchange products and sz_i sz_j are recognised
        # separately.
        exch = np.zeros((N, N))     # exch[a, b]: coefficient of X(a, b) = c^+_au c_bu c^+_bd c_ad
        zz = np.zeros((N, N))
        nud = np.zeros(N)           # n_up (1 - n_down) terms of sisj((i,),(i,))
        for c, strs, elems in rest:
            if strs == ["c_dagger_c", "c_dagger_c"]:
                (a1, s1), (b1, s1b) = elems[0]
                (a2, s2), (b2, s2b) = elems[1]
                if _is_up(s1) == _is_up(s1b) and _is_up(s2) == _is_up(s2b) and _is_up(s1) != _is_up(s2) \
                        and a1 == b2 and b1 == a2 and a1 != b1:
                    a, b = (a1, b1) if _is_up(s1) else (b1, a1)   # X(a, b): up hop b -> a, down hop a -> b
                    exch[a, b] += c
                    continue
            elif strs == ["sz", "sz"]:
                zz[elems[0][0][0], elems[1][0][0]] += c
                continue
            elif strs == ["n", "1_n"] and elems[0][0][0] == elems[1][0][0] and _is_up(elems[0][0][1]) \
                    and not _is_up(elems[1][0][1]):
                nud[elems[0][0][0]] += c
                continue
            raise NotImplementedError(f"the expectation of {_print_term(strs, elems)} needs the generic operator "
                                      "engine")
        sec = _capi.Sector(N, int(self.n_up[0]), int(self.n_down[0]), _capi.ED_HUBBARD, t=np.zeros((N, N)),
                           U=np.zeros(N))
        x = sec.from_ref(torch.tensor(np.asarray(psi, dtype=np.float64), device="cuda"))
        pairs = [(J, K) for J in range(1, N + 1) for K in range(1, N + 1)]
        raw, _ = sec.rdm_raw(x, pairs=pairs, flags=3)
        q = raw.reshape(N, N, 6)   # q[J-1][K-1]: see ed_rdm
        val = const * float(psi @ psi)
        for i in range(N):
            for j in range(N):
                if i == j:
                    val += tu[i, i] * q[i, i, 0] + td[i, i] * q[i, i, 2] + U[i] * q[i, i, 3]
                    val += nud[i] * (q[i, i, 0] - q[i, i, 3]) + zz[i, i] * q[i, i, 1]
                else:
                    # <c^+_i c_j>: the hop j -> i of q[i][j] (up: column 0, down: column 4)
                    val += tu[i, j] * q[i, j, 0] + td[i, j] * q[i, j, 4] + zz[i, j] * q[i, j, 1]
                    # q[i][j][5] = -<c^+_ju c_iu c^+_id c_jd> (static_rq.f90:345-383, up hop i -> j with the
                    # down hop j -> i) = -<X(j, i)>, X(a, b) = c^+_au c_bu c^+_bd c_ad
                    val += -exch[j, i] * q[i, j, 5]
        return float(val)

    # ------------------------------------------------------------ derived
    @property
    def to_matrix(self):
        """Row i = the operator applied to basis state i (the reference fills
        H[i,:] that way, _operators.py:267-279)."""
        self._check_basis()
        n = self.nstates
        M = np.zeros((n, n))
        e = np.zeros(n)
        for i in range(n):
            e[i] = 1.0
            M[i, :] = self._apply(e)
            e[i] = 0.0
        return M

    def lanczos(self, maxstep=200, acc_lcz=1.0e-8, neigen=1, init_states=None):
        """The reference's plain Lanczos on this operator (_operators.py:283-322):
        random uniform[-0.5,0.5) start unless init_states, checks every 5
        steps that the first neigen Ritz values moved by less than acc_lcz
        (mean norm), at most maxstep steps.  Runs the three-term recurrence on
        the GPU sector product and rebuilds the Ritz vectors by a second pass.
        Returns (ek[:neigen], psi) with psi [nstates, neigen]."""
        from ..core import lanczos as LZ
        torch = _torch()
        self._check_basis()
        sec, const = self._sector_of()
        if const != 0.0:
            raise NotImplementedError("lanczos of an operator with an identity term: shift the energies instead")
        v = (np.random.random(self.nb_selected) - 0.5) if not isinstance(init_states, np.ndarray) else init_states
        x = sec.from_ref(torch.tensor(np.asarray(v, dtype=np.float64), device="cuda"))
        rule = _OperatorRule(acc_lcz, neigen)
        r = LZ.lanczos_plain(sec, x, maxstep, rule=rule, check_every=5, nvec=neigen)
        self._lcz = r
        ek = np.asarray(r.ritz[:neigen])
        psi = np.stack([sec.to_ref(p).cpu().numpy() for p in r.psis], axis=1)
        return ek, psi

    @property
    def alpha(self):
        return None if self._lcz is None else self._lcz.alpha

    @property
    def beta(self):
        return None if self._lcz is None else self._lcz.beta


class _OperatorRule:
    """Convergence test of Operators.lanczos (_operators.py:297-314): the mean
    change of the first neigen Ritz values between checks below acc."""

    wants_vectors = False

    def __init__(self, acc: float, neigen: int):
        self.acc = float(acc)
        self.neigen = int(neigen)
        self.prev = np.full(self.neigen, 100.0)
        self.converged = False
        self.ndeg = 1

    def __call__(self, val, step=0):
        ek = np.full(self.neigen, 100.0)
        k = min(self.neigen, len(val))
        ek[:k] = val[:k]
        if np.linalg.norm(ek - self.prev) / self.neigen < self.acc:
            self.converged = True
        self.prev = ek
        return self.converged


def _print_from_string(string, args):
    if string == "c_dagger_c":
        return f"c^\\dagger_{{{args[0][0]},{args[0][1]}}}c_{{{args[1][0]},{args[1][1]}}}"
    if string == "c_dagger":
        return f"c^\\dagger_{{{args[0][0]},{args[0][1]}}}"
    if string == "c":
        return f"c_{{{args[0][0]},{args[0][1]}}}"
    if string == "n":
        return f"n_{{{args[0][0]},{args[0][1]}}}"
    if string == "1_n":
        return f"(1 - n_{{{args[0][0]},{args[0][1]}}})"
    if string == "sz":
        return f"S^z_{{{args[0][0]}}}"
    if string == "sisj":
        return f"S_{{{args[0][0]}}}S_{{{args[1][0]}}}"
    if string == "splus":
        return f"S^+_{{{args[0][0]}}}"
    if string == "sminus":
        return f"S^-_{{{args[0][0]}}}"
    return ""


def _print_term(strs, elems):
    return "".join(_print_from_string(s, e) for s, e in zip(strs, elems)) or "id."
