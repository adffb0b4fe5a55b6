"""Operators API (pyhub/core/_operators.py, pyhub/tools/operators.py,
pyhub/tools/models.py) on the GPU sector product and RDM kernel, against a
Jordan-Wigner construction of the same operators in the oracle (modes: down
sites then up sites, so a same-spin hop counts only same-spin modes between
its ends: the ANTICOM signs of operators.f90).

Tolerances: H @ psi, to_matrix and <O> 1e-12 relative (FP64); Lanczos E0 1e-9
against dense diagonalisation, Ritz vector overlap 1 - 1e-8."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _jw(norb, sec):
    """Fock-space builders restricted to the (N_up, N_down) sector."""
    import scipy.sparse as sp
    c = O._jw_ops(2 * norb)
    cs = {"dn": lambda i: c[i], "up": lambda i: c[norb + i]}
    idx = np.array([O._fock_index(norb, int(u), int(d)) for d in sec.bdn for u in sec.bup], dtype=np.int64)
    I = sp.identity(2 ** (2 * norb), format="csr")

    def restrict(M):
        return M[idx][:, idx].toarray()

    def cdc(i, si, j, sj):
        return cs[si](i).T @ cs[sj](j)

    def n(i, s):
        return cdc(i, s, i, s)

    def sz(i):
        return 0.5 * (n(i, "up") - n(i, "dn"))

    def sisj(i, j):
        if i == j:
            return 2 * (n(i, "up") @ (I - n(i, "dn"))) / 2 + sz(i) @ sz(i)
        return -(cdc(i, "up", j, "up") @ cdc(j, "dn", i, "dn") + cdc(i, "dn", j, "dn") @ cdc(j, "up", i, "up")) / 2 \
            + sz(i) @ sz(j)

    return restrict, cdc, n, sisj


def _case(norb=6, nu=3, nd=2, seed=0):
    rng = np.random.default_rng(seed)
    t = rng.standard_normal((norb, norb))
    t = 0.5 * (t + t.T)
    U = rng.uniform(1, 5, norb)
    sec = O.Sector(norb, nu, nd)
    psi = rng.standard_normal(sec.dim)
    return t, U, sec, psi / np.linalg.norm(psi)


def test_fermi_hubbard_apply_matrix_lanczos(edlib):
    from pyhub_gb300.core.basis import Basis
    from pyhub_gb300.tools.models import fermi_hubbard
    t, U, sec, psi = _case()
    restrict, cdc, n, _ = _jw(6, sec)
    Hd = O.jw_hubbard_sector(sec, t, U)
    H = fermi_hubbard(t, U)
    H.set_basis(Basis(6, (3, 2)))
    y = H @ psi
    assert np.linalg.norm(y - Hd @ psi) <= 1e-12 * np.linalg.norm(Hd @ psi)
    assert abs(H.avg(psi) - psi @ Hd @ psi) <= 1e-12 * abs(psi @ Hd @ psi)
    M = H.to_matrix
    assert np.abs(M - Hd.T).max() <= 1e-12 * np.abs(Hd).max()
    # complex vectors: real and imaginary parts separately, as the reference does
    z = psi + 1j * np.roll(psi, 3)
    assert np.linalg.norm((H @ z) - Hd @ z) <= 1e-12 * np.linalg.norm(Hd @ z)
    val, vec = np.linalg.eigh(Hd)
    np.random.seed(1)
    ek, V = H.lanczos(maxstep=200, acc_lcz=1e-12, neigen=1)
    assert abs(ek[0] - val[0]) < 1e-9
    assert abs(float(V[:, 0] @ vec[:, 0])) > 1 - 1e-8
    # scalar shift and sums keep the Hubbard form
    H2 = 2.0 * H + 1.5
    H2.set_basis(Basis(6, (3, 2)))
    assert np.linalg.norm(H2 @ psi - (2 * Hd @ psi + 1.5 * psi)) <= 1e-12 * np.linalg.norm(Hd @ psi)


def test_one_body_and_density_averages(edlib):
    from pyhub_gb300.core.basis import Basis
    from pyhub_gb300.tools.operators import c_dagger_c, n
    t, U, sec, psi = _case(seed=2)
    restrict, cdc, nn, _ = _jw(6, sec)
    B = Basis(6, (3, 2))
    for (i, j, s) in [(0, 3, "up"), (4, 1, "down"), (2, 2, "up"), (5, 0, "d")]:
        op = c_dagger_c((i, s), (j, s))
        op.set_basis(B)
        ss = "up" if s in ("up", "u") else "dn"
        ref = psi @ restrict(cdc(i, ss, j, ss)) @ psi
        assert abs(op.avg(psi) - ref) <= 1e-12, (i, j, s)
    op = n((3, "up")) * n((3, "down")) + 0.5 * n((1, "down")) - 2.0 * c_dagger_c((2, "up"), (5, "up"))
    op.set_basis(B)
    ref = psi @ restrict(nn(3, "up") @ nn(3, "dn") + 0.5 * nn(1, "dn") - 2.0 * cdc(2, "up", 5, "up")) @ psi
    assert abs(op.avg(psi) - ref) <= 1e-12


@pytest.mark.parametrize("pair", [(0, 1), (2, 5), (4, 4)])
def test_sisj_average(edlib, pair):
    from pyhub_gb300.core.basis import Basis
    from pyhub_gb300.tools.operators import sisj
    t, U, sec, psi = _case(norb=6, nu=3, nd=3, seed=5)
    restrict, _, _, S = _jw(6, sec)
    op = sisj((pair[0],), (pair[1],))
    op.set_basis(Basis(6, (3, 3)))
    ref = psi @ restrict(S(*pair)) @ psi
    assert abs(op.avg(psi) - ref) <= 1e-12 * max(1.0, abs(ref)), (op.avg(psi), ref)


def test_heisenberg_model_average_and_application(edlib):
    """heisenberg(J) on the fermionic basis: <H> through the RDM route, and H psi
    on the generic operator engine, both against the Jordan-Wigner S_i.S_j; the
    Hubbard model on a basis of two up-particle numbers on the engine, against
    the oracle's HPROD of each sector."""
    from pyhub_gb300.core.basis import Basis
    from pyhub_gb300.tools.models import fermi_hubbard, heisenberg
    norb = 4
    J = O.ring(norb, 1.0)
    sec = O.Sector(norb, 2, 2)
    rng = np.random.default_rng(7)
    psi = rng.standard_normal(sec.dim)
    restrict, _, _, S = _jw(norb, sec)
    ref = sum(J[i, j] * (psi @ restrict(S(i, j)) @ psi) for i in range(norb) for j in range(norb))
    H = heisenberg(J)
    H.set_basis(Basis(norb, (2, 2)))
    assert abs(H.avg(psi) - ref) <= 1e-12 * max(1.0, abs(ref))
    hpsi = sum(J[i, j] * (restrict(S(i, j)) @ psi) for i in range(norb) for j in range(norb))
    np.testing.assert_allclose(H @ psi, hpsi, rtol=0, atol=1e-12 * max(1.0, np.abs(hpsi).max()))
    t = O.ring(norb, -1.0)
    F = fermi_hubbard(t, 2.0)
    F.set_basis(Basis(norb, ([1, 2], [2])))
    x = rng.standard_normal(F.nstates)
    y = F @ x
    # the vector is [down string][up string] over up strings of 1 then 2 particles: each sector's part
    n1, n2, nd = O.binom(norb, 1), O.binom(norb, 2), O.binom(norb, 2)
    X, Y = x.reshape(nd, n1 + n2), y.reshape(nd, n1 + n2)
    for nu, cols in ((1, slice(0, n1)), (2, slice(n1, n1 + n2))):
        ref_s = O.hprod_hubbard(O.Sector(norb, nu, 2), t, 2.0, X[:, cols].reshape(-1))
        np.testing.assert_allclose(Y[:, cols].reshape(-1), ref_s, rtol=0, atol=1e-12)
