"""The generic operator engine (ed_ops_apply) against the oracle's
restatement of operators.x, and the Operators API on the paths it opens.

Tolerances: the engine and the oracle do the same operations in the same
order (factor images are exact: +-x, x/2 or 0; the term sum is one multiply
and one add per term), so their results agree bit for bit.  API results are
checked against the oracle to 1e-12 (Lanczos eigenvalues to 1e-8 of the
dense spectrum)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

CODES_1 = [2, 4, 10, 11]          # one site, one spin
SPACES = [(4, [2], [2]), (4, [1, 2, 3], [0, 2]), (5, [0, 1, 2, 3, 4, 5], [2, 3]), (6, [3, 2], [1, 4])]


def _random_terms(rng, norb, nterms=6, maxlen=3):
    terms = []
    for _ in range(nterms):
        ops = []
        for _ in range(int(rng.integers(1, maxlen + 1))):
            code = int(rng.choice([1, 2, 4, 5, 6, 7, 9, 10, 11, 12, 3]))
            i, j = (int(v) for v in rng.integers(1, norb + 1, size=2))
            s1, s2 = (int(v) for v in rng.integers(1, 3, size=2))
            ops.append((code, i, s1, j, s2))
        terms.append((float(rng.normal()), ops))
    return terms


@pytest.mark.parametrize("space", SPACES)
def test_engine_matches_oracle_bit_for_bit(edlib, space):
    import torch
    norb, nups, ndns = space
    sp = edlib.OpSpace(norb, nups, ndns)
    bup, bdn = O.ops_space(norb, nups, ndns)
    assert (sp.nsup, sp.nsdn) == (len(bup), len(bdn))
    rng = np.random.default_rng(norb * 7 + len(nups))
    psi = rng.normal(size=sp.nstates)
    x = torch.tensor(psi, device="cuda")
    for trial in range(6):
        terms = _random_terms(rng, norb)
        got = sp.apply(terms, x).cpu().numpy()
        ref = O.ops_apply_ref(norb, nups, ndns, terms, psi)
        np.testing.assert_array_equal(got, ref, err_msg=str(terms))
    # every code alone, every site and spin
    for code in (1, 2, 4, 5, 6, 7, 9, 10, 11, 12):
        for i in range(1, norb + 1):
            for s1 in (1, 2):
                t = [(1.0, [(code, i, s1, (i % norb) + 1, 3 - s1)])]
                np.testing.assert_array_equal(sp.apply(t, x).cpu().numpy(), O.ops_apply_ref(norb, nups, ndns, t, psi))


def test_engine_refuses_bad_terms(edlib):
    import torch
    sp = edlib.OpSpace(4, [2], [2])
    x = torch.zeros(sp.nstates, dtype=torch.float64, device="cuda")
    for bad in ([(1.0, [(8, 1, 1, 2, 1)])], [(1.0, [(1, 5, 1, 1, 1)])], [(1.0, [(2, 1, 3, 0, 0)])],
                [(1.0, [(13, 1, 1, 0, 0)])]):
        with pytest.raises(edlib.EDError):
            sp.apply(bad, x)
    with pytest.raises(edlib.EDError):
        edlib.OpSpace(4, [2, 2], [1])


def test_operators_generic_paths_match_oracle(edlib):
    from pyhub_gb300.core.basis import Basis
    from pyhub_gb300.tools import operators as OP
    norb = 4
    nups, ndns = [1, 2], [1, 2]
    op = (OP.c_dagger((0, 'u')) * OP._c((2, 'u')) - 0.7 * OP.splus((1,)) * OP.sminus((3,))
          + 0.3 * OP.sz((2,)) + OP.c_dagger_c((0, 'u'), (1, 'd')) + 1.25)
    op.set_basis(Basis(norb, hilbert=(nups, ndns)))
    terms = op._encode()
    rng = np.random.default_rng(5)
    psi = rng.normal(size=op.nstates)
    ref = O.ops_apply_ref(norb, nups, ndns, terms, psi)
    np.testing.assert_allclose(op @ psi, ref, rtol=0, atol=1e-12)
    assert abs(op.avg(psi) - psi @ ref) < 1e-12
    # complex vectors: real and imaginary parts separately, as the reference does
    z = psi + 1j * rng.normal(size=op.nstates)
    np.testing.assert_allclose(op @ z, O.ops_apply_ref(norb, nups, ndns, terms, z.real)
                               + 1j * O.ops_apply_ref(norb, nups, ndns, terms, z.imag), atol=1e-12)
    # to_matrix: row i = the operator applied to basis state i, with the basis-element routines (their sz is
    # SZ_BASIS, + S^z, where the vector routines' SZ_OPE gives (n_down - n_up)/2)
    M = op.to_matrix
    bterms = op._encode(basis_mode=True)
    assert [c for _, ops in bterms for c, *_ in ops].count(12) == 1
    for i in (0, 7, op.nstates - 1):
        e = np.zeros(op.nstates)
        e[i] = 1.0
        np.testing.assert_allclose(M[i], O.ops_apply_ref(norb, nups, ndns, bterms, e), atol=1e-12)
    # comparisons: the diagonal, up string outer and down string inner
    diag = np.array([M[d * op.nsup + u, d * op.nsup + u] for u in range(op.nsup) for d in range(op.nsdown)])
    assert (op == 1.25) == [bool(np.isclose(v, 1.25)) for v in diag]
    assert (op > 1.0) == [bool(v > 1.0) for v in diag]
    assert "| <H>" in op.bit_repr()
    # a selection: input zero outside it, output read on it
    sel = np.array([1, 4, 9, 17, 30])
    ops = op[sel]
    v = rng.normal(size=len(sel))
    full = np.zeros(op.nstates)
    full[sel] = v
    np.testing.assert_allclose(ops @ v, O.ops_apply_ref(norb, nups, ndns, terms, full)[sel], atol=1e-12)
    np.testing.assert_allclose(ops.to_matrix, M[np.ix_(sel, sel)], atol=1e-12)


def test_operators_lanczos_on_several_sectors(edlib):
    """The reference's operator Lanczos on a Hubbard Hamiltonian over a basis
    of several (N_up, N_down) sectors: its lowest eigenvalue is the lowest of
    the sectors' dense spectra."""
    from pyhub_gb300.core.basis import Basis
    from pyhub_gb300.tools import operators as OP
    norb = 4
    t = O.ring(norb)
    H = 0
    for i in range(norb):
        for j in range(norb):
            if t[i, j] != 0:
                H = H + t[i, j] * (OP.c_dagger_c((i, 'u'), (j, 'u')) + OP.c_dagger_c((i, 'd'), (j, 'd')))
        H = H + 4.0 * OP.n((i, 'u')) * OP.n((i, 'd'))
    nups, ndns = [1, 2], [2]
    H.set_basis(Basis(norb, hilbert=(nups, ndns)))
    np.random.seed(3)
    ek, psi = H.lanczos(maxstep=120, acc_lcz=1e-10, neigen=1)
    e_ref = min(np.linalg.eigvalsh(O.dense_h(lambda v: O.hprod_hubbard(O.Sector(norb, nu, 2), t, 4.0, v),
                                             O.binom(norb, nu) * O.binom(norb, 2)))[0] for nu in nups)
    assert abs(ek[0] - e_ref) < 1e-8
    r = H @ psi[:, 0] - ek[0] * psi[:, 0]
    assert np.linalg.norm(r) < 1e-5 * np.linalg.norm(psi[:, 0])
