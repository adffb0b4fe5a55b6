"""Operator algebra with the reference's API (pyhub/core/_operators.py:10-705),
evaluated on the GPU.

The reference keeps an operator as a sum of products of elementary
operators (c_dagger_c, c_dagger, c, n, 1_n, sz, splus, sminus, id.) and
applies it to a vector by writing the term list and the vector to
operators.h5 and running the Fortran program operators.x
(`__call__`, :145-205; `to_matrix`, :254-281; `lanczos`, :283-322).  Here the
same term list is kept in memory and applied on the device:

* Hubbard form on one (N_up, N_down) sector -- sums of c^+_{i s} c_{j s}
  (both spins with the same coefficient matrix), n_{i s} and
  n_{i up} n_{i down} terms and the identity -- runs as the H*v of a sector
  built from the recognised (t, U).  operators.x applies c^+_J c_K with the
  same KINOP/ANTICOM signs and the same (d-1)*NSUP+u index as HPROD
  (operators.f90:1-59), so the results are the reference's.
* Everything else -- any product of the elementary operators, on a basis of
  several listed particle numbers or on a selection of its states -- runs on
  the generic operator engine (ed_ops_apply), which restates operators.x
  routine by routine: the factors of a product act in list order, the first
  one first, and a factor whose result leaves the listed particle numbers
  drops it, as the Fortran does.  Its `sz` element is SZ_OPE
  (operators.f90:223-248), which multiplies by (n_down - n_up)/2; products
  sz*sz, as sisj builds them, are the usual S^z_i S^z_j.  to_matrix, the
  comparisons and bit_repr use the reference's basis-element routines
  (operators_basis.f90), whose sz (SZ_BASIS) is +S^z.
* Expectation values of one-body terms of either spin, densities,
  n_{i up} n_{i down} and the spin correlation sisj((i,),(j,)) on one sector
  go through the fused RDM kernel (ed_rdm).
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
                mul.set_basis(Basis(self.nb_sites, self.hilbert, self.order), selected=self.selected)
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

    def __rtruediv__(self, other):
        # the reference forwards to a __rdiv__ it does not define (_operators.py:127-128)
        raise TypeError("a number cannot be divided by an operator")

    def __req__(self, other):
        return self.__eq__(other)

    def __iter__(self):
        """Each term as its own operator: coeff * the product of its elements
        (_operators.py:238-242)."""
        iter_op = []
        for i, coeff in enumerate(self.coeff):
            iter_op.append(coeff * self.__multiplemul__([_operator_from_string(st, elem) for st, elem in
                                                         zip(self.str_index[i], self.elem_index[i])]))
        return iter_op.__iter__()

    def __multiplemul__(self, other):
        mul = Operators._idt()
        for o in other:
            mul *= o
        return mul

    def __getitem__(self, index):
        """The operator on a selection of basis states (_operators.py:131-147):
        vectors then hold the selected states' components, and products are
        the reference's: the input is zero outside the selection and the
        output is read on it."""
        if isinstance(index, (list, np.ndarray)):
            sel = np.asarray(index, dtype=int)
            other = Operators.empty_operator()
            other.coeff, other.elem_index, other.str_index = self.coeff, self.elem_index, self.str_index
            other.set_basis(Basis(self.nb_sites, self.hilbert, self.order), selected=sel)
            return other
        return None

    def __delitem__(self):
        # the reference deletes the operator's group of operators.h5 (_operators.py:251-253); nothing is
        # stored here
        return None

    # ------------------------------------------------------------ comparisons with a number
    def _compare(self, other, op):
        """[op(<s|O|s>, other) for every basis state s] in the reference's order:
        the selected states, or every up string for every down string
        (_operators.py:555-705)."""
        if not isinstance(other, (float, int)):
            raise TypeError(f"an operator compares with a number, not {type(other)}")
        self._check_basis()
        diag = self._diagonal()
        if self.selected is None:
            # the reference loops posu outer, posd inner; the diagonal is in d*nsup + u order
            diag = diag.reshape(self.nsdown, self.nsup).T.reshape(-1)
        return [bool(op(v, other)) for v in diag]

    def __eq__(self, other):
        return self._compare(other, lambda v, o: np.isclose(v, o))

    def __ne__(self, other):
        return [not e for e in self.__eq__(other)]

    def __ge__(self, other):
        return self._compare(other, lambda v, o: v >= o)

    def __gt__(self, other):
        return self._compare(other, lambda v, o: v > o)

    def __le__(self, other):
        return self._compare(other, lambda v, o: v <= o)

    def __lt__(self, other):
        return self._compare(other, lambda v, o: v < o)

    __hash__ = None

    # ------------------------------------------------------------ file bookkeeping of the reference
    @property
    def filename_operators(self):
        return "operators.h5"

    @property
    def index_str(self):
        return str(getattr(self, "_index", 1)).rjust(6, "0")

    @property
    def file_size(self):
        """Size of the reference's operators.h5; nothing is written here."""
        return 0.0

    def _write_operator(self, max_len_ope=40):
        # the reference writes the term list to operators.h5 (_operators.py:395-462); here the list is
        # encoded per product (_encode)
        self.op2write = False
        self.max_len_ope = max_len_ope

    def exec_operators(self):
        # the reference runs operators.x (_operators.py:208-222); products run in process
        self._check_basis()

    def _set_basis_elem(self, posu, posd, up, down):
        # the reference writes one basis element to operators.h5 for the basis-element mode; the
        # comparisons and bit_repr take the diagonal directly
        return None

    @property
    def T(self):
        # unimplemented in the reference (_operators.py:380-382): None
        return None

    @property
    def dagger(self):
        return self.T

    def bit_repr(self):
        """The basis states (the selected ones when there is a selection) with
        <s|O|s>, in the reference's layout (_operators.py:474-508)."""
        self._check_basis()
        select = self.selected if isinstance(self.selected, (list, np.ndarray)) else list(range(self.nstates))
        diag = self._diagonal()
        string = '-' * (3 * (self.nb_sites + 4)) + '\n'
        string += 'empty        : 0\nuparrow      : 1\ndownarrow    :-1\nupdoawnarrow : 2\n'
        string += '-' * (3 * (self.nb_sites + 4)) + '\n'
        string += 'index | bit' + ' ' * (3 * (self.nb_sites - 1) - 1) + ' | <H> ' + '\n'
        string += '------|----' + '-' * (3 * (self.nb_sites - 1) - 1) + '-|-----' + '\n'
        for k, index in enumerate(self.basis[select]):
            up, down = self.decompose(int(index))
            string += "{:4d}  |".format(int(index))
            for i in range(self.nb_sites):
                u, d = (up >> i) & 1, (down >> i) & 1
                string += ' 0 ' if (not u and not d) else (' 1 ' if (u and not d) else ('-1 ' if (d and not u) else ' 2 '))
            string += f' | {np.around(diag[k], 4)}' + '\n'
        return string

    def find_stable_space(self):
        # "Experimental function, do not use!" in the reference (_operators.py:510-553)
        raise NotImplementedError("find_stable_space is experimental in the reference and not provided")

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

    def _one_sector(self) -> bool:
        """One (N_up, N_down) sector and no selection: the sector fast paths apply."""
        return self.selected is None and len(self.n_up) == 1 and len(self.n_down) == 1

    # ------------------------------------------------------------ generic engine
    def _encode(self, basis_mode: bool = False):
        """The term list as _write_operator encodes it (_operators.py:420-462):
        [(coeff, [(code, site1, spin1, site2, spin2), ...])], sites 1-based,
        spin 1 = up, 2 = down.  basis_mode: the reference's basis-element
        routines (operators_basis.f90), which differ from the vector routines
        in one place: their sz multiplies by +S^z (SZ_BASIS, engine code 12)
        where SZ_OPE gives (n_down - n_up)/2."""
        codes = {"n": 2, "id.": 3, "1_n": 4, "sz": 12 if basis_mode else 5, "splus": 6, "sminus": 7, "sisj": 8,
                 "c_dagger": 10, "c": 11}
        terms = []
        for c, strs, elems in zip(self.coeff, self.str_index, self.elem_index):
            ops = []
            for st, idx in zip(strs, elems):
                site1 = site2 = spin1 = spin2 = 0
                try:
                    site1 = idx[0][0] + 1
                    site2 = idx[1][0] + 1
                except (IndexError, TypeError):
                    pass
                try:
                    spin1 = 1 if _is_up(idx[0][1]) else 2
                    spin2 = 1 if _is_up(idx[1][1]) else 2
                except (IndexError, TypeError):
                    pass
                if st == "c_dagger_c":
                    code = 1 if idx[0][1] == idx[1][1] else 9
                elif st in codes:
                    code = codes[st]
                else:
                    raise NotImplementedError(f"operator element {st!r}")
                ops.append((code, site1, spin1, site2, spin2))
            terms.append((float(c), ops))
        return terms

    def _space(self):
        key = (self.nb_sites, tuple(int(n) for n in self.n_up), tuple(int(n) for n in self.n_down))
        sp = getattr(self, "_opspace", None)
        if sp is None or sp[0] != key:
            sp = (key, _capi.OpSpace(self.nb_sites, key[1], key[2]))
            self._opspace = sp
        return sp[1]

    def _apply_generic_full(self, x_full: np.ndarray, basis_mode: bool = False) -> np.ndarray:
        """The operator applied to a vector of the whole space (the reference's
        psi/input dataset), on the generic engine; basis_mode: with the
        semantics of the basis-element routines (to_matrix, the comparisons,
        bit_repr)."""
        torch = _torch()
        sp = self._space()
        x = torch.tensor(np.asarray(x_full, dtype=np.float64), device="cuda")
        return sp.apply(self._encode(basis_mode), x).cpu().numpy()

    def _embed(self, psi: np.ndarray) -> np.ndarray:
        """psi of the selected states placed in the whole space (zeros elsewhere),
        as __call__ writes its input (_operators.py:155-160)."""
        if self.selected is None:
            return np.asarray(psi, dtype=np.float64)
        full = np.zeros(self.nstates)
        full[np.asarray(self.selected, dtype=int)] = psi
        return full

    def _restrict(self, v: np.ndarray) -> np.ndarray:
        return v if self.selected is None else v[np.asarray(self.selected, dtype=int)]

    def _diagonal(self) -> np.ndarray:
        """<s|O|s> of every basis state (the selected ones when there is a
        selection), in basis order: what the reference's basis-element mode
        returns as avg_value one state at a time (_operators.py:474-508)."""
        states = np.arange(self.nstates) if self.selected is None else np.asarray(self.selected, dtype=int)
        out = np.zeros(len(states))
        e = np.zeros(self.nstates)
        for k, s_ in enumerate(states):
            e[s_] = 1.0
            out[k] = (self._apply_generic_full(e, basis_mode=True))[s_]
            e[s_] = 0.0
        return out

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
            elif strs == ["c_dagger_c"] and elems[0][0][1] == elems[0][1][1]:
                # same spin label: C_DAGGER_C; different labels (even 'u' and 'up') are the spin-flip
                # C_DAGGER_C_UNRES, as the reference's operator file encodes them (_operators.py:438-439)
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
        if not self._one_sector() or self._hubbard() is None:
            return self._restrict(self._apply_generic_full(self._embed(psi)))
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
        if not self._one_sector():
            full = self._embed(psi)
            return float(full @ self._apply_generic_full(full))
        if self._hubbard() is not None:
            return float(psi @ self._apply(psi))
        try:
            return self._rdm_expectation(psi)
        except NotImplementedError:
            return float(psi @ self._restrict(self._apply_generic_full(self._embed(psi))))

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
        H[i,:] that way, _operators.py:254-281); on a selection, the rows and
        columns of the selected states."""
        self._check_basis()
        if not self._one_sector() or self._hubbard() is None:
            states = np.arange(self.nstates) if self.selected is None else np.asarray(self.selected, dtype=int)
            M = np.zeros((len(states), len(states)))
            e = np.zeros(self.nstates)
            for i, s_ in enumerate(states):
                e[s_] = 1.0
                M[i, :] = self._apply_generic_full(e, basis_mode=True)[states]
                e[s_] = 0.0
            return M
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
        h = self._hubbard() if self._one_sector() else None
        if h is None or h[2] != 0.0:
            return self._lanczos_generic(maxstep, acc_lcz, neigen, init_states)
        sec, const = self._sector_of()
        v = (np.random.random(self.nb_selected) - 0.5) if not isinstance(init_states, np.ndarray) else init_states
        x = sec.from_ref(torch.tensor(np.asarray(v, dtype=np.float64), device="cuda"))
        rule = _OperatorRule(acc_lcz, neigen)
        r = LZ.lanczos_plain(sec, x, maxstep, rule=rule, check_every=5, nvec=neigen)
        self._lcz = r
        ek = np.asarray(r.ritz[:neigen])
        psi = np.stack([sec.to_ref(p).cpu().numpy() for p in r.psis], axis=1)
        return ek, psi

    def _lanczos_generic(self, maxstep, acc_lcz, neigen, init_states):
        """The reference's loop as written (_operators.py:325-364), with the
        products on the generic engine: plain three-term recurrence, checks
        every 5 steps on the first neigen Ritz values, at most maxstep - 5
        steps, psi = V^T Vk[:, :neigen]."""
        from scipy.linalg import eigh_tridiagonal
        v = (np.random.random(self.nb_selected) - .5) if not isinstance(init_states, np.ndarray) else init_states
        v = np.asarray(v, dtype=np.float64)
        alpha, beta, vecs = [], [np.linalg.norm(v)], []
        v = v / beta[0]
        v0 = np.zeros(self.nb_selected)
        nstep, ek, ekm1 = 0, np.full(neigen, 100.), np.full(neigen, 0.)
        Vk = np.zeros((0, 0))
        nadd = 5
        while nstep < maxstep - nadd and not np.linalg.norm(ek[:neigen] - ekm1) / neigen < acc_lcz:
            ekm1 = np.copy(ek[:neigen])
            for _ in range(nadd):
                vecs.append(v)
                v2 = self @ v
                alpha.append(v2 @ v)
                v2 = v2 - alpha[-1] * v - beta[-1] * v0
                beta.append(np.linalg.norm(v2))
                v0 = v
                v = v2 / beta[-1]
                nstep += 1
            ek, Vk = eigh_tridiagonal(alpha, beta[1:nstep], eigvals_only=False, select='a')
        self._lcz = type("GenericLanczos", (), {"alpha": np.array(alpha), "beta": np.array(beta[1:])})()
        psi = np.array(vecs[:len(alpha)]).T @ Vk[:, :neigen]
        return ek[:neigen], psi

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


def _operator_from_string(string, args):
    """One elementary operator from its name and indices (_operators.py:708-733)."""
    op = Operators(*args)
    if string not in ("c_dagger_c", "c_dagger", "c", "n", "1_n", "sz", "sisj", "splus", "sminus", "id."):
        raise ValueError(f"unknown operator element {string!r}")
    op.str_index = [[string]]
    if string == "id.":
        op.elem_index = [[()]]
    return op


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
