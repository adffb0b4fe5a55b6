"""The generic operator engine's oracle and term encoding (host only).

The oracle restates operators.x routine by routine (oracle.ops_apply_ref);
here it is checked against identities that hold in the reference's own
conventions on the full Fock space (every particle number listed): a factor
list acts first factor first, c then c^+ on one mode is n, c^+ then c is
1 - n, c_j then c^+_i is the hop C_DAGGER_C(i, j), and the spin-flip hops
and S^+/S^- equal their c/c^+ products.  The encoding of Operators terms is
checked against the rules of _write_operator (_operators.py:420-462)."""
import numpy as np
import pytest

from oracle import oracle as O

NORB = 4
FULL = list(range(NORB + 1))


@pytest.fixture(scope="module")
def psi():
    bup, bdn = O.ops_space(NORB, FULL, FULL)
    return np.random.default_rng(0).normal(size=len(bup) * len(bdn))


def _ap(ops, psi, nups=FULL, ndns=FULL):
    return O.ops_apply_ref(NORB, nups, ndns, [(1.0, ops)], psi)


@pytest.mark.parametrize("sp", [1, 2])
def test_density_identities(psi, sp):
    for i in range(1, NORB + 1):
        n = _ap([(2, i, sp, 0, 0)], psi)
        np.testing.assert_array_equal(_ap([(1, i, sp, i, sp)], psi), n)          # c^+_i c_i = n_i
        np.testing.assert_array_equal(_ap([(11, i, sp, 0, 0), (10, i, sp, 0, 0)], psi), n)
        np.testing.assert_array_equal(_ap([(10, i, sp, 0, 0), (11, i, sp, 0, 0)], psi), _ap([(4, i, sp, 0, 0)], psi))
        np.testing.assert_array_equal(n + _ap([(4, i, sp, 0, 0)], psi), psi)       # n + (1 - n) = 1


@pytest.mark.parametrize("sp", [1, 2])
def test_hop_is_annihilation_then_creation(psi, sp):
    for i in range(1, NORB + 1):
        for j in range(1, NORB + 1):
            if i != j:
                np.testing.assert_array_equal(_ap([(11, j, sp, 0, 0), (10, i, sp, 0, 0)], psi),
                                              _ap([(1, i, sp, j, sp)], psi))


def test_spin_flips(psi):
    for i in range(1, NORB + 1):
        np.testing.assert_array_equal(_ap([(6, i, 0, 0, 0)], psi), _ap([(11, i, 2, 0, 0), (10, i, 1, 0, 0)], psi))
        np.testing.assert_array_equal(_ap([(7, i, 0, 0, 0)], psi), _ap([(11, i, 1, 0, 0), (10, i, 2, 0, 0)], psi))
        for j in range(1, NORB + 1):
            for spj, spi in ((1, 2), (2, 1)):
                np.testing.assert_array_equal(_ap([(9, i, 0, j, spj)], psi),
                                              _ap([(11, j, spj, 0, 0), (10, i, spi, 0, 0)], psi))


def test_sz_is_sz_ope(psi):
    """SZ_OPE multiplies by ((1 - n_up) - (1 - n_down)) / 2 = (n_down - n_up) / 2."""
    for i in range(1, NORB + 1):
        ref = 0.5 * (_ap([(2, i, 2, 0, 0)], psi) - _ap([(2, i, 1, 0, 0)], psi))
        np.testing.assert_allclose(_ap([(5, i, 0, 0, 0)], psi), ref, rtol=0, atol=1e-15)


def test_sz_basis_is_minus_sz_ope(psi):
    """The basis-element sz (SZ_BASIS, engine code 12) multiplies by +S^z."""
    for i in range(1, NORB + 1):
        np.testing.assert_array_equal(_ap([(12, i, 0, 0, 0)], psi), -_ap([(5, i, 0, 0, 0)], psi))


def test_terms_restart_from_psi_and_drop_unlisted_sectors():
    bup, bdn = O.ops_space(NORB, [1, 2], [2])
    psi = np.random.default_rng(1).normal(size=len(bup) * len(bdn))
    terms = [(2.0, [(10, 1, 1, 0, 0)]), (-0.5, [(2, 3, 2, 0, 0)]), (1e-15, [(4, 1, 1, 0, 0)])]
    out = O.ops_apply_ref(NORB, [1, 2], [2], terms, psi)
    a = O.ops_apply_ref(NORB, [1, 2], [2], [(1.0, [(10, 1, 1, 0, 0)])], psi)
    b = O.ops_apply_ref(NORB, [1, 2], [2], [(1.0, [(2, 3, 2, 0, 0)])], psi)
    np.testing.assert_array_equal(out, 2.0 * a + (-0.5) * b)
    # c^+_up takes 1-particle up strings into the 2-particle block and 2-particle strings to 3
    # particles, which are not listed and are dropped: nothing lands in the 1-particle block
    n1 = O.binom(NORB, 1)
    blocks = a.reshape(len(bdn), len(bup))
    assert np.all(blocks[:, :n1] == 0.0) and np.any(blocks[:, n1:] != 0.0)


def test_operator_terms_encode_as_the_reference_writes_them():
    from pyhub_gb300.tools import operators as OP
    op = (OP.c_dagger_c((0, 'u'), (2, 'u')) + 2.0 * OP.n((1, 'd')) * OP._n((3, 'u'))
          - OP.sz((2,)) * OP.splus((1,)) + OP.c_dagger((0, 'd')) * OP._c((1, 'd'))
          + OP.c_dagger_c((0, 'u'), (1, 'd')) + OP.c_dagger_c((0, 'u'), (1, 'up')) + 1.5)
    enc = op._encode()
    assert enc == [(1.0, [(1, 1, 1, 3, 1)]), (2.0, [(2, 2, 2, 0, 0), (4, 4, 1, 0, 0)]),
                   (-1.0, [(5, 3, 0, 0, 0), (6, 2, 0, 0, 0)]), (1.0, [(10, 1, 2, 0, 0), (11, 2, 2, 0, 0)]),
                   (1.0, [(9, 1, 1, 2, 2)]), (1.0, [(9, 1, 1, 2, 1)]), (1.5, [(3, 0, 0, 0, 0)])]
    # iterating yields each term as its own operator, coefficient included
    terms = list(op)
    assert len(terms) == op.nb_ope and [t.coeff for t in terms][1] == [2.0]


def test_operator_selection_and_comparison_arguments():
    from pyhub_gb300.core.basis import Basis
    from pyhub_gb300.tools import operators as OP
    op = OP.n((0, 'u')) + OP.n((1, 'd'))
    op.set_basis(Basis(4, hilbert=([1, 2], [1, 2])))
    sel = op[np.array([0, 3, 5])]
    assert list(sel.selected) == [0, 3, 5] and sel.nb_selected == 3
    with pytest.raises(TypeError):
        op == None  # noqa: E711
    with pytest.raises(TypeError):
        1.0 / op
    assert op.T is None and op.dagger is None and op.file_size == 0.0


def _jw_restricted(norb, bup, bdn):
    """Jordan-Wigner operators of the Fock space restricted to the product of
    the up and down string lists (index d * len(bup) + u)."""
    c = O._jw_ops(2 * norb)
    cs = {"d": lambda i: c[i], "u": lambda i: c[norb + i]}
    idx = np.array([O._fock_index(norb, int(u), int(d)) for d in bdn for u in bup], dtype=np.int64)

    def restrict(M):
        return M[idx][:, idx].toarray()

    def cdc(i, si, j, sj):
        return cs[si](i).T @ cs[sj](j)

    return restrict, cdc


def test_oracle_models_match_jordan_wigner():
    """operators.x's restatement applied to fermi_hubbard on a basis of two up
    numbers and to heisenberg(J) equals the Jordan-Wigner operators; the two
    model builders' products are bilinears, for which the reference's
    conventions and Jordan-Wigner agree."""
    from pyhub_gb300.tools.models import fermi_hubbard, heisenberg
    norb = 4
    rng = np.random.default_rng(11)
    t = O.ring(norb, -1.0)
    t[0, 2] = t[2, 0] = 0.4
    F = fermi_hubbard(t, 2.5)
    bup, bdn = O.ops_space(norb, [1, 2], [2])
    restrict, cdc = _jw_restricted(norb, bup, bdn)
    Hjw = 0
    for i in range(norb):
        for j in range(norb):
            if t[i, j] != 0:
                Hjw = Hjw + t[i, j] * (cdc(i, "u", j, "u") + cdc(i, "d", j, "d"))
        Hjw = Hjw + 2.5 * (cdc(i, "u", i, "u") @ cdc(i, "d", i, "d"))
    x = rng.normal(size=len(bup) * len(bdn))
    np.testing.assert_allclose(O.ops_apply_ref(norb, [1, 2], [2], F._encode(), x), restrict(Hjw) @ x,
                               rtol=0, atol=1e-13)
    J = O.ring(norb, 1.0)
    bup, bdn = O.ops_space(norb, [2], [2])
    restrict, cdc = _jw_restricted(norb, bup, bdn)
    n = lambda i, s: cdc(i, s, i, s)  # noqa: E731
    sz = lambda i: 0.5 * (n(i, "u") - n(i, "d"))  # noqa: E731
    Sjw = 0
    for i in range(norb):
        for j in range(norb):
            if J[i, j] != 0:
                Sjw = Sjw + J[i, j] * (-(cdc(i, "u", j, "u") @ cdc(j, "d", i, "d")
                                         + cdc(i, "d", j, "d") @ cdc(j, "u", i, "u")) / 2 + sz(i) @ sz(j))
    x = rng.normal(size=len(bup) * len(bdn))
    np.testing.assert_allclose(O.ops_apply_ref(norb, [2], [2], heisenberg(J)._encode(), x), restrict(Sjw) @ x,
                               rtol=0, atol=1e-13)
