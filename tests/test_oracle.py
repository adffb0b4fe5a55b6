"""CPU tests of the oracle: basis order, rank, and the sign conventions of
the restated HPROD / RDM / GF routines against an independent Jordan-Wigner
construction, plus physics identities.  No GPU."""
import itertools

import numpy as np
import pytest

from oracle import oracle as O


@pytest.mark.parametrize("no,ne", [(4, 2), (8, 4), (12, 6), (12, 5), (14, 7), (16, 8), (6, 0), (6, 6), (10, 3)])
def test_hilbert_order_is_lexicographic_subsets(no, ne):
    # compute_basis.f90 HILBERT enumerates subsets of bit positions in lexicographic order
    assert np.array_equal(O.hilbert(no, ne), O.hilbert_py(no, ne))


def test_hilbert_python_restatement_of_move_bmove():
    """A line-by-line Python restatement of HILBERT/MOVE/BMOVE agrees with the C one."""
    def move(s, posf):
        a = 1 << (posf - 1)
        return (s ^ a) ^ (1 << posf)

    def bmove(no, s):
        nsm = 0
        while (s >> (no - nsm - 1)) & 1:
            nsm += 1
        sf = s - sum(1 << (no - i) for i in range(1, nsm + 1))
        posle = no
        while not (sf >> (posle - 1)) & 1:
            posle -= 1
        sf -= 1 << (posle - 1)
        sm = sf + sum(1 << (posle - 1 + i) for i in range(1, nsm + 2))
        return sm, posle + 1 + nsm

    for no, ne in [(6, 3), (9, 4), (11, 5)]:
        ns = O.binom(no, ne)
        b = [sum(1 << (i - 1) for i in range(1, ne + 1))]
        pos = ne
        while len(b) < ns:
            while pos < no and len(b) < ns:
                b.append(move(b[-1], pos))
                pos += 1
            if len(b) < ns:
                s, pos = bmove(no, b[-1])
                b.append(s)
        assert np.array_equal(np.array(b, dtype=np.uint32), O.hilbert(no, ne))


@pytest.mark.parametrize("no,ne", [(8, 4), (12, 5), (14, 7), (16, 8), (20, 3)])
def test_rank_inverts_hilbert(no, ne):
    b = O.hilbert(no, ne)
    idx = np.random.default_rng(0).choice(len(b), size=min(300, len(b)), replace=False)
    for i in idx:
        assert O.rank(no, ne, int(b[i])) == i


def test_kinop_anticom_definitions():
    # KINOP (funcmod.f90:18-27): site POS <-> bit NORB-POS
    norb = 6
    s = 0b101100  # sites 1,3,4 occupied
    assert O.lib().orc_kinop(norb, s, 1, 2) == 0b011100
    assert O.lib().orc_kinop(norb, s, 2, 5) == 0       # site 2 empty
    assert O.lib().orc_kinop(norb, s, 1, 3) == 0       # site 3 occupied
    assert O.lib().orc_kinop(norb, s, 3, 3) == s       # J==K occupied: diagonal
    # ANTICOM: (-1)^(occupied sites before POS)
    assert O.lib().orc_anticom(norb, 1, s) == 1.0
    assert O.lib().orc_anticom(norb, 2, s) == -1.0
    assert O.lib().orc_anticom(norb, 4, s) == 1.0
    assert O.lib().orc_anticom(norb, 6, s) == -1.0


HUB = [(2, 1, 1), (3, 1, 2), (4, 2, 2), (4, 1, 3), (5, 2, 3), (5, 3, 3), (6, 3, 3), (6, 2, 4), (6, 0, 2)]


@pytest.mark.parametrize("case", HUB)
@pytest.mark.parametrize("sym", [True, False])
def test_hubbard_restatement_equals_jordan_wigner(case, sym):
    n, nu, nd = case
    rng = np.random.default_rng(n * 7 + nu)
    t = rng.standard_normal((n, n))
    if sym:
        t = t + t.T
    U = rng.uniform(0, 5, n)
    sec = O.Sector(n, nu, nd)
    H_or = O.dense_h(lambda v: O.hprod_hubbard(sec, t, U, v), sec.dim)
    H_jw = O.jw_hubbard_sector(sec, t, U)
    assert np.abs(H_or - H_jw).max() <= 1e-13 * max(1.0, np.abs(H_jw).max())


@pytest.mark.parametrize("case", [(4, 2, 2), (6, 3, 3), (7, 3, 2), (8, 4, 4)])
def test_fast_hprod_equals_reference_loop(case):
    n, nu, nd = case
    rng = np.random.default_rng(1)
    t = rng.standard_normal((n, n))
    t = t + t.T
    U = rng.uniform(0, 5, n)
    sec = O.Sector(n, nu, nd)
    x = rng.standard_normal(sec.dim)
    a = O.hprod_hubbard(sec, t, U, x)
    b = O.hprod_hubbard(sec, t, U, x, fast=True, nthreads=2)
    assert np.linalg.norm(a - b) <= 1e-14 * np.linalg.norm(a)


def test_pair_sample_sums_to_full_product():
    n, nu, nd = 6, 3, 2
    t = O.ring(n)
    sec = O.Sector(n, nu, nd)
    x = np.random.default_rng(2).standard_normal(sec.dim)
    full = O.hprod_hubbard(sec, t, 0.0, x)
    y = np.zeros(sec.dim)
    pairs = [(J, K) for J in range(1, n + 1) for K in range(1, n + 1)]
    O.hprod_hubbard_pairs(sec, t, pairs, x, y)
    assert np.allclose(y, full, rtol=0, atol=1e-13)


@pytest.mark.parametrize("case", [(8, 4, 4), (9, 4, 3), (10, 3, 6)])
def test_threaded_reference_loop_is_bit_identical(case):
    """The host-threaded reference loop timed as the CPU baseline adds every
    element's terms in the serial loop's order: equal bit for bit."""
    norb, nu, nd = case
    rng = np.random.default_rng(norb + nu)
    t = rng.standard_normal((norb, norb))
    t = 0.5 * (t + t.T)
    sec = O.Sector(norb, nu, nd)
    pairs = [(J, K) for J in range(1, norb + 1) for K in range(1, norb + 1) if J != K]
    x = rng.standard_normal(sec.dim)
    y1, y2 = np.zeros(sec.dim), np.zeros(sec.dim)
    O.hprod_hubbard_pairs(sec, t, pairs, x, y1, nthreads=1)
    O.hprod_hubbard_pairs(sec, t, pairs, x, y2, nthreads=5)
    for J in range(1, norb + 1):
        O.hprod_hubbard_udiag(sec, J, 1.5 + J, x, y1, nthreads=1)
        O.hprod_hubbard_udiag(sec, J, 1.5 + J, x, y2, nthreads=3)
    assert np.array_equal(y1, y2)


@pytest.mark.parametrize("n", [2, 4, 6])
def test_heisenberg_restatement_equals_jordan_wigner(n):
    rng = np.random.default_rng(n)
    J = rng.standard_normal((n, n))
    J = J + J.T
    H_or = O.dense_h(lambda v: O.hprod_heis(n, J, v), O.binom(n, n // 2))
    H_jw = O.jw_heis_sector(n, J)
    assert np.abs(H_or - H_jw).max() <= 1e-13 * np.abs(H_jw).max()
    x = rng.standard_normal(len(H_or))
    assert np.allclose(O.hprod_heis(n, J, x, fast=True), H_or @ x, rtol=0, atol=1e-12)


def test_heisenberg_spectrum_bipartite_vs_triangle():
    """hprod_heis.f90:44-45 pairs ANTICOM(J,dn)*ANTICOM(K,new_dn) with the down
    hop K->J, which flips the sign of the transverse exchange.  On bipartite
    clusters that is a sublattice gauge transformation (same spectrum as the
    physical sum_JK J_JK S_J.S_K); on a triangle it is not."""
    for n in (4, 6):
        J = O.ring(n, 1.0)
        a = np.linalg.eigvalsh(O.jw_heis_sector(n, J))
        b = np.linalg.eigvalsh(O.jw_heis_sector(n, J, physical=True))
        assert np.allclose(a, b, atol=1e-12)
    J = np.ones((3, 3)) - np.eye(3)
    a = np.linalg.eigvalsh(O.jw_heis_sector(3, J))
    b = np.linalg.eigvalsh(O.jw_heis_sector(3, J, physical=True))
    assert not np.allclose(a, b)


def test_c1_ring_identities():
    """L=8 ring, U=4: reference-rule Lanczos = dense ED; Tr gamma = N;
    sum t gamma + sum U <n n> = E0 on the exact eigenvector; S^2 = 0."""
    sec = O.Sector(8, 4, 4)
    t, U = O.ring(8), 4.0
    H = O.dense_h(lambda v: O.hprod_hubbard(sec, t, U, v, fast=True), sec.dim)
    val, vec, ndeg = O.exact_diag(H)
    assert ndeg == 1
    v0 = np.random.default_rng(0).uniform(-0.5, 0.5, sec.dim)
    r = O.lanczos_ref(lambda v: O.hprod_hubbard(sec, t, U, v, fast=True), v0, 600, 1e-8)
    assert r["converged"] and abs(r["eigenvalues"][0] - val[0]) < 1e-9
    psi = vec[:, 0]
    g = O.one_rdm(sec, psi)
    assert abs(np.trace(g["up"]) - 4) < 1e-12 and abs(np.trace(g["down"]) - 4) < 1e-12
    ni = O.two_rdm_ni(sec, psi)
    e = np.sum(t * (g["up"] + g["down"])) + U * ni.sum()
    assert abs(e - val[0]) < 1e-11
    sm = O.j_spin(sec, psi)
    assert abs(sm.sum()) < 1e-10
    assert np.allclose(sm, sm.T)


def test_gf_start_vectors_match_jordan_wigner():
    """LCZ_{H,E}_{UP,DOWN} start vectors equal c|psi> / c^+|psi> built in the
    Fock space with down modes ordered before up modes."""
    from oracle.oracle import _fock_index, _jw_ops
    n, nu, nd = 4, 2, 1
    sec = O.Sector(n, nu, nd)
    rng = np.random.default_rng(4)
    psi = rng.standard_normal(sec.dim)
    c = _jw_ops(2 * n)
    fock = np.zeros(1 << (2 * n))
    idx = [_fock_index(n, int(u), int(d)) for d in sec.bdn for u in sec.bup]
    fock[idx] = psi
    for kind in ("h_up", "h_down", "e_up", "e_down"):
        sec1, st = O.gf_start(kind, sec, n, psi)
        idx1 = [_fock_index(n, int(u), int(d)) for d in sec1.bdn for u in sec1.bup]
        for pos in range(1, n + 1):
            mode = (n + pos - 1) if kind.endswith("up") else (pos - 1)
            op = c[mode] if kind.startswith("h") else c[mode].T
            out = op @ fock
            assert np.allclose(out[idx1], st[pos - 1], atol=1e-14)


def test_boltzmann_zero_temperature():
    w = O.boltzmann(np.array([-3.0, -2.0, -1.0]), 0.0, 1)
    assert np.array_equal(w, [1.0])
    w = O.boltzmann(np.array([-3.0, -2.0, -1.0]), 0.0, 2)
    assert np.array_equal(w, [1.0, 0.0])
    w = O.boltzmann(np.array([-3.0, -2.9, 50.0]), 1.0, 1)
    assert len(w) == 2 and np.allclose(w, [1.0, np.exp(-0.1)])


def test_operator_algebra_recognises_hubbard_form():
    """Operators API on the host: the Hubbard model's term list maps back to
    its (t, U); sisj stays outside the Hubbard form (CPU, no GPU needed)."""
    from pyhub_gb300.core.basis import Basis
    from pyhub_gb300.tools.models import fermi_hubbard
    from pyhub_gb300.tools.operators import c_dagger_c, n, sisj
    rng = np.random.default_rng(0)
    t = rng.standard_normal((5, 5))
    U = rng.uniform(1, 4, 5)
    H = fermi_hubbard(t, U) + 0.5
    H.set_basis(Basis(5, (2, 3)))
    tt, UU, const = H._hubbard()
    assert np.array_equal(tt, t) and np.array_equal(UU, U) and const == 0.5
    assert (2.0 * H)._hubbard()[0][1, 2] == 2.0 * t[1, 2]
    S = sisj((0,), (3,))
    S.set_basis(Basis(5, (2, 3)))
    assert S._hubbard() is None and len(S._classify()[4]) == 3
    op = c_dagger_c((0, "up"), (1, "up")) + n((2, "down"))
    op.set_basis(Basis(5, (2, 3)))
    assert op._hubbard() is None          # spin-dependent one-body terms: averages only
    assert str(c_dagger_c((0, "u"), (1, "u"))) == "1.0*c^\\dagger_{0,u}c_{1,u}"



@pytest.mark.parametrize("no,ne", [(10, 5), (12, 6), (16, 8), (32, 16)])
def test_unrank_inverts_rank(no, ne):
    rng = np.random.default_rng(no)
    n = O.binom(no, ne)
    for r in rng.integers(0, n, 300):
        s = O.unrank(no, ne, int(r))
        assert bin(s).count("1") == ne and O.rank(no, ne, s) == int(r)
    if no <= 16:
        b = O.hilbert(no, ne)
        assert all(O.unrank(no, ne, i) == int(b[i]) for i in range(0, n, max(1, n // 500)))


def test_hashvec_matches_c():
    L = O.lib()
    idx = [0, 1, 7, 12345, 601080389, 2 ** 31 + 5]
    for kind in (0, 1):
        v = O.hashvec(idx, 3, kind)
        assert all(L.orc_hashval(i, 3, kind) == v[q] for q, i in enumerate(idx))
    assert set(np.unique(O.hashvec(np.arange(1000), 1, 1))) <= set(range(-3, 4))


@pytest.mark.parametrize("norb,lattice", [(10, (5, 2)), (12, (4, 3))])
def test_heis_rows_equal_full_restatement(norb, lattice):
    """The output-side row form of the Heisenberg HPROD equals the scatter
    restatement bit for bit on every row (real and integer inputs, with
    diagonal J terms present)."""
    J = np.abs(O.square_pbc(*lattice, 1.0))
    J[0, 0], J[3, 3] = 0.7, -0.2
    J[1, 5] = 0.3   # an asymmetric extra term
    n = O.binom(norb, norb // 2)
    for kind in (0, 1):
        x = O.hashvec(np.arange(n), 5, kind)
        y = O.hprod_heis(norb, J, x)
        yr, ab = O.hprod_heis_rows(norb, J, np.arange(n), 5, kind)
        assert np.array_equal(yr, y)
        assert np.all(ab >= np.abs(y) - 1e-12)


def test_j_spin_heis_rows_equal_masked_restatement():
    """J_SPIN with the bra restricted to sampled rows equals the full
    restatement with a bra that is zero off those rows."""
    norb = 12
    n = O.binom(norb, norb // 2)
    rows = np.sort(np.random.default_rng(3).choice(n, 150, replace=False))
    for kind in (0, 1):
        bra = np.zeros(n)
        bra[rows] = O.hashvec(rows, 11, kind)
        ket = O.hashvec(np.arange(n), 12, kind)
        full = O.j_spin_heis(norb, bra, ket)           # Python view: SMATRIX transposed
        pairs = [(J, K) for J in range(1, norb + 1) for K in range(1, norb + 1)]
        got, ab = O.j_spin_heis_rows(norb, rows, 11, 12, kind, pairs)
        ref = np.array([full[K - 1, J - 1] for (J, K) in pairs])
        assert np.allclose(got, ref, rtol=0, atol=1e-13 * max(1.0, ab.max()))
        if kind == 1:
            assert np.array_equal(got, ref)


def test_threaded_full_hubbard_loop_is_bit_identical():
    sec = O.Sector(8, 4, 3)
    rng = np.random.default_rng(4)
    t = rng.standard_normal((8, 8))
    U = rng.uniform(0, 5, 8)
    x = rng.standard_normal(sec.dim)
    assert np.array_equal(O.hprod_hubbard_mt(sec, t, U, x, nthreads=3), O.hprod_hubbard(sec, t, U, x))
    sec = O.Sector(8, 4, 4)
    x = rng.standard_normal(sec.dim)
    assert np.array_equal(O.hprod_hubbard_mt(sec, t, U, x, nthreads=2), O.hprod_hubbard(sec, t, U, x))


def test_self_energy_restatement_vanishes_without_interaction():
    """U = 0: the SPGF_ED poles give G = G0 exactly, so the restated
    self_energy is zero; with U > 0 it is not."""
    norb = 5
    t = O.ring(norb)
    t[0, 2] = t[2, 0] = -0.4
    ek, Vk = np.linalg.eigh(t)
    for U, zero in ((0.0, True), (2.5, False)):
        sec = O.Sector(norb, 2, 2)
        H = O.dense_h(lambda v: O.hprod_hubbard(sec, t, U, v), sec.dim)
        e, v = np.linalg.eigh(H)
        sp = O.spgf_ed(sec, t, U, [v[:, 0]], norb)
        diag = O.lehmann_gf_diag(sec, t, U, v[:, 0], e[0], norb)
        pos, Q = diag["up"]["greater"]
        assert np.allclose(sp["Q_greater_up"][:, :, 0], Q) and np.allclose(sp["positions_greater_up"] - e[0], pos)
        S = O.self_energy_ref(Vk, ek, e[:1], [1.0], sp, 0.37, 0.1, True)
        mag = np.abs(S["up"]).max()
        assert (mag < 1e-9) if zero else (mag > 1e-3), (U, mag)


def _uijkl(rng, n, density=0.4):
    Ul = rng.standard_normal((n,) * 4) * (rng.random((n,) * 4) < density)
    Ul = 0.5 * (Ul + np.einsum("ijkl->jilk", Ul))   # the symmetry the reference requires (core_solver.py:143)
    Ul[1, 0] = 0.0                                  # a (J,K) pair gated off by UPARTIAL
    return Ul


@pytest.mark.parametrize("case", [(4, 2, 2), (4, 2, 1), (5, 2, 3), (5, 3, 3)])
def test_uijkl_restatement_equals_jordan_wigner(case):
    """IS_ULOC=3: the HPROD restatement (index order UL(J,K,M,N) =
    U[N-1,M-1,K-1,J-1], UPARTIAL gate) equals the Fock-space construction,
    and DBL_OCC of TWO_RDM equals <ket|c+_K c_J c+_N c_M|bra> for K<=J, N<=M."""
    n, nu, nd = case
    rng = np.random.default_rng(n * 10 + nu)
    sec = O.Sector(n, nu, nd)
    t = rng.standard_normal((n, n))
    t = t + t.T
    Ul = _uijkl(rng, n)
    H = O.jw_hubbard_uijkl_sector(sec, t, Ul)
    Hd = O.dense_h(lambda v: O.hprod_hubbard_uijkl(sec, t, Ul, v), sec.dim)
    assert np.abs(H - Hd).max() <= 1e-13 * max(1.0, np.abs(H).max())
    bra, ket = rng.standard_normal(sec.dim), rng.standard_normal(sec.dim)
    dbl, ni = O.two_rdm_dbl_occ(sec, bra, ket)
    for J in range(1, n + 1):
        for K in range(1, J + 1):
            for M in range(1, n + 1):
                for N in range(1, M + 1):
                    v = O.jw_two_body(sec, bra, ket, J, K, M, N)
                    assert abs(dbl[J - 1, K - 1, M - 1, N - 1] - v) <= 1e-12, (J, K, M, N)
                    assert dbl[K - 1, J - 1, N - 1, M - 1] == dbl[J - 1, K - 1, M - 1, N - 1]
    assert np.array_equal(ni, [dbl[j, j, j, j] for j in range(n)])
