"""GPU parity of the loops built on H*v -- RDMs, Green's-function start
vectors and poles, the Lanczos variants -- and of the drop-in Python API,
against the CPU oracle.

Tolerances: RDM sums of FP64 states 1e-12 absolute; GF start vectors
bit-exact (a signed copy); E0 1e-10 against dense diagonalisation; G(w) on a
grid within 1e-6 of the exact Lehmann sum (continued fraction run to the
Krylov dimension of small sectors).
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _state(norb, nu, nd, seed):
    rng = np.random.default_rng(seed)
    t = rng.standard_normal((norb, norb))
    t = np.triu(t) + np.triu(t, 1).T
    U = rng.uniform(0.5, 6.0, norb)
    return t, U, rng


@pytest.mark.parametrize("case", [(4, 2, 2), (6, 3, 3), (6, 2, 4), (7, 3, 2), (8, 4, 4), (8, 3, 4)])
def test_rdm_matches_oracle(edlib, case):
    import torch
    from pyhub_gb300.core.reduced_quantities import all_pairs, assemble_hubbard
    norb, nu, nd = case
    t, U, rng = _state(norb, nu, nd, sum(case))
    osec = O.Sector(norb, nu, nd)
    sec = edlib.Sector(norb, nu, nd, edlib.ED_HUBBARD, t=t, U=U)
    bra = rng.standard_normal(osec.dim)
    bra /= np.linalg.norm(bra)
    for ket in (bra, rng.standard_normal(osec.dim)):
        b = sec.from_ref(torch.tensor(bra, device="cuda"))
        k = sec.from_ref(torch.tensor(ket, device="cuda"))
        flags = 2 | (1 if nu != nd else 0)
        raw, _ = sec.rdm_raw(b, k if ket is not bra else None, pairs=all_pairs(norb), flags=flags)
        gu, gd, ni, sm = assemble_hubbard(raw, norb, nu, nd)
        ref = O.one_rdm(osec, bra, ket)
        assert np.abs(gu - ref["up"]).max() < 1e-12
        assert np.abs(gd - ref["down"]).max() < 1e-12
        assert np.abs(ni - O.two_rdm_ni(osec, bra, ket)).max() < 1e-12
        assert np.abs(sm - O.j_spin(osec, bra, ket)).max() < 1e-12


@pytest.mark.parametrize("norb", [4, 6, 8, 10])
def test_heisenberg_rdm_matches_oracle(edlib, norb):
    import torch
    from pyhub_gb300.core.reduced_quantities import all_pairs, assemble_heisenberg
    rng = np.random.default_rng(norb)
    J = O.ring(norb, 1.0)
    sec = edlib.Sector(norb, norb // 2, 0, edlib.ED_HEISENBERG, J=J)
    bra = rng.standard_normal(sec.dim)
    ket = rng.standard_normal(sec.dim)
    raw, _ = sec.rdm_raw(sec.from_ref(torch.tensor(bra, device="cuda")), sec.from_ref(torch.tensor(ket, device="cuda")),
                         pairs=all_pairs(norb))
    got = assemble_heisenberg(raw, norb)
    assert np.abs(got - O.j_spin_heis(norb, bra, ket)).max() < 1e-11


@pytest.mark.parametrize("case", [(5, 2, 3), (6, 3, 3), (6, 3, 2)])
def test_gf_start_vectors_exact(edlib, case):
    import torch
    norb, nu, nd = case
    t, U, rng = _state(norb, nu, nd, 3)
    osec = O.Sector(norb, nu, nd)
    psi = rng.standard_normal(osec.dim)
    src = edlib.Sector(norb, nu, nd, edlib.ED_HUBBARD, t=t, U=U)
    pd = src.from_ref(torch.tensor(psi, device="cuda"))
    for kind in ("h_up", "h_down", "e_up", "e_down"):
        osec1, ref = O.gf_start(kind, osec, norb, psi)
        if osec1.dim == 0:
            continue
        dst = edlib.Sector(norb, osec1.nup, osec1.ndn, edlib.ED_HUBBARD, t=t, U=U)
        for site in range(1, norb + 1):
            out = torch.full((dst.n,), float("nan"), dtype=torch.float64, device="cuda")
            edlib.gf_start(src, dst, kind, site, pd, out)
            got = dst.to_ref(out).cpu().numpy()
            assert np.array_equal(got, ref[site - 1])


def test_gf_start_sites_equals_per_site(edlib):
    """ed_gf_start_sites (all sites in one launch, vectors a stride apart)
    writes exactly what ed_gf_start writes site by site."""
    import torch
    norb, nu, nd = 6, 3, 2
    t, U, rng = _state(norb, nu, nd, 5)
    src = edlib.Sector(norb, nu, nd, edlib.ED_HUBBARD, t=t, U=U)
    psi = src.from_ref(torch.tensor(rng.standard_normal(src.dim), device="cuda"))
    for kind, (du, dd) in (("h_up", (-1, 0)), ("e_down", (0, 1))):
        dst = edlib.Sector(norb, nu + du, nd + dd, edlib.ED_HUBBARD, t=t, U=U)
        stride = dst.n + 32
        out = torch.full((norb * stride,), float("nan"), dtype=torch.float32, device="cuda")
        edlib.gf_start_sites(src, dst, kind, list(range(1, norb + 1)), psi, out, stride)
        for site in range(1, norb + 1):
            ref = torch.zeros(dst.n, dtype=torch.float32, device="cuda")
            edlib.gf_start(src, dst, kind, site, psi, ref)
            got = out[(site - 1) * stride: (site - 1) * stride + dst.n]
            assert torch.equal(dst.to_ref(got), dst.to_ref(ref)), (kind, site)


def test_gf_poles_match_lehmann(edlib):
    """Small 6-site cluster: the continued-fraction poles give the exact
    Lehmann G_ij(w) of SPGF_ED on a frequency grid, and fh.gf -- which, like
    the reference's compute_gf, passes the poles through Pole.clean(wtol=1e-8),
    rounding positions to 5 decimals -- equals the Lehmann poles put through
    the same clean()."""
    from pyhub_gb300.solver import FermiHubbard
    from pyhub_gb300.tools.pole import Pole
    norb = 6
    t = O.ring(norb)
    t[0, 3] = t[3, 0] = -0.3
    U = 3.0
    fh = FermiHubbard(norb, 3, 3, t, U)
    fh.kernel(max_lcz=300, acc_lcz=1e-13, compute_rq=False)   # dim 400 > 300: Lanczos path
    fh.spgf(nsteps=400)
    osec = O.Sector(norb, 3, 3)
    H = O.dense_h(lambda v: O.hprod_hubbard(osec, t, U, v, fast=True), osec.dim)
    e, v = np.linalg.eigh(H)
    assert abs(fh.e0 - e[0]) < 1e-11
    ref = O.lehmann_gf_diag(osec, t, U, v[:, 0], e[0], norb)
    w = np.linspace(-8, 8, 301)
    eta = 0.05
    for spin in ("up", "down"):
        for i in range(norb):
            for j in range(norb):
                exact = 0
                cleaned = []
                raw = 0
                for part in ("greater", "lesser"):
                    pos, Q = ref[spin][part]
                    exact = exact + O.poles_eval(pos, Q[i] * Q[j], w, eta)
                    cleaned.append(Pole({"positions": pos, "weights": Q[i] * Q[j]}).clean(wtol=1.e-8))
                    p_, w_ = fh._spgf[0][spin][part].pole(i, j)
                    raw = raw + O.poles_eval(p_, w_, w, eta)
                assert np.abs(raw - exact).max() < 1e-7, (spin, i, j)
                got = fh.gf[spin][i, j].retarded(w, eta=eta)
                assert np.abs(got - Pole.sum(cleaned).retarded(w, eta=eta)).max() < 1e-6, (spin, i, j)


def test_fermi_hubbard_api_c1(edlib):
    """L=8 ring, U=4, N_up=N_down=4: the drop-in API against dense ED and the
    oracle's RDM routines on the exact ground state."""
    from pyhub_gb300.solver import FermiHubbard
    t = O.ring(8)
    fh = FermiHubbard(8, 4, 4, t, 4.0)
    fh.kernel(max_lcz=600, acc_lcz=1e-8)
    osec = O.Sector(8, 4, 4)
    H = O.dense_h(lambda v: O.hprod_hubbard(osec, t, 4.0, v, fast=True), osec.dim)
    e, v = np.linalg.eigh(H)
    assert abs(fh.e0 - e[0]) < 1e-10
    assert fh.is_lanczos and fh.nb_deg >= 0
    psi = fh.psi0
    assert abs(abs(psi @ v[:, 0]) - 1) < 1e-8
    ref = O.one_rdm(osec, v[:, 0])
    assert np.abs(fh.one_rdm["up"] - ref["up"]).max() < 1e-6
    assert np.abs(fh.ni - O.two_rdm_ni(osec, v[:, 0])).max() < 1e-6
    assert np.abs(fh.spin_cor_matrix - O.j_spin(osec, v[:, 0])).max() < 1e-6
    assert abs(fh.e_one_body + np.sum(fh.ni * 4.0) - fh.e0) < 1e-7


def test_fermi_hubbard_small_sector_exact_diag(edlib):
    from pyhub_gb300.solver import FermiHubbard
    t = O.ring(4)
    fh = FermiHubbard(4, 2, 1, t, 2.0)
    fh.kernel(nb_comp_states=2, store_H=True)
    osec = O.Sector(4, 2, 1)
    H = O.dense_h(lambda v: O.hprod_hubbard(osec, t, 2.0, v), osec.dim)
    assert np.array_equal(fh.H, H)
    e = np.linalg.eigvalsh(H)
    assert np.allclose(fh.e, e, atol=1e-12)
    fh.set_state(1)
    assert abs(fh.e0 - e[1]) < 1e-12


def test_heisenberg_api_ring(edlib):
    from pyhub_gb300.solver import Heisenberg
    n = 12
    J = O.ring(n, 1.0)
    h = Heisenberg(n, J)
    h.kernel(max_lcz=200)
    Hd = O.dense_h(lambda v: O.hprod_heis(n, J, v, fast=True), O.binom(n, n // 2))
    e, v = np.linalg.eigh(Hd)
    assert abs(h.e0 - e[0]) < 1e-10
    sm = O.j_spin_heis(n, v[:, 0])
    assert np.abs(h.spin_cor_matrix - sm).max() < 1e-6


@pytest.mark.parametrize("dt", ["f64", "f32"])
def test_three_term_lanczos_matches_full(edlib, dt):
    import torch
    from pyhub_gb300.core import lanczos as LZ
    t = O.square_pbc(3, 3)
    sec = edlib.Sector(9, 4, 5, edlib.ED_HUBBARD, t=t, U=np.full(9, 4.0))
    td = torch.float64 if dt == "f64" else torch.float32
    v0 = LZ.start_vector(sec, 3, dtype=td)
    a = LZ.lanczos_full(sec, v0, 80, td)
    b = LZ.lanczos_plain(sec, v0, 80, nvec=1)
    tol = 1e-9 if dt == "f64" else 1e-4
    assert abs(a.ritz[0] - b.ritz[0]) < tol
    if dt == "f64":
        # without reorthogonalisation an FP32 basis loses orthogonality within a few
        # dozen steps, so only the FP64 Ritz vector is compared
        ov = float((a.psi * b.psis[0]).sum().item())
        assert abs(abs(ov) - 1) < 1e-8


@pytest.mark.parametrize("layout", ["hubbard", "heisenberg"])
def test_three_term_kept_basis_equals_replay(edlib, layout):
    """The three-term Lanczos with its basis kept (Ritz vectors by one pass
    over the kept rows), with a cap of 12 rows (rows run out mid-run: rotating
    vectors, then a replay on the same schedule) and without keeping (replay)
    runs the same recurrence.  The kept rows subtract u_{k-1} before u_k while
    the rotating vectors take them in ring order, so the paths agree to
    rounding: alpha/beta to 1e-12 relative, Ritz vectors to 1e-10 (FP64, 40
    steps).  Padded (Hubbard) and unpadded (Heisenberg) layouts."""
    import torch
    from pyhub_gb300.core import lanczos as LZ
    if layout == "hubbard":
        sec = edlib.Sector(9, 4, 5, edlib.ED_HUBBARD, t=O.square_pbc(3, 3), U=np.full(9, 4.0))
    else:
        sec = edlib.Sector(16, 8, 0, edlib.ED_HEISENBERG, J=O.square_pbc(4, 4, 1.0))
    v0 = LZ.start_vector(sec, 5, dtype=torch.float64)
    runs = [LZ.lanczos_plain(sec, v0, 40, nvec=2, keep=k) for k in (True, 12, False)]
    for r in runs[1:]:
        assert r.steps == runs[0].steps == 40
        assert np.allclose(r.alpha, runs[0].alpha, rtol=1e-12, atol=0)
        assert np.allclose(r.beta, runs[0].beta, rtol=1e-12, atol=0)
        for p, q in zip(r.psis, runs[0].psis):
            assert float(torch.linalg.vector_norm(p - q)) < 1e-10


def test_heisenberg_lattice_rdm_and_plain_mixed_ground_state(edlib):
    """4x4 periodic Heisenberg (dim 12,870): spin correlations of the row
    layout vs the oracle's J_SPIN on random bra/ket (all pairs, 1e-11); the
    three-term mixed-precision ground state (FP32 then FP64 refinement, four
    vectors) vs the full-reorthogonalisation FP64 one (|dE0| < 1e-9); and the
    bond-energy identity E0 = sum_{J!=K} J_JK (q1 - q0) on its vector."""
    import torch
    from pyhub_gb300.core import lanczos as LZ
    from pyhub_gb300.core.reduced_quantities import all_pairs, assemble_heisenberg
    norb = 16
    J = O.square_pbc(4, 4, 1.0)
    sec = edlib.Sector(norb, 8, 0, edlib.ED_HEISENBERG, J=J)
    rng = np.random.default_rng(4)
    bra = rng.standard_normal(sec.dim)
    ket = rng.standard_normal(sec.dim)
    raw, _ = sec.rdm_raw(sec.from_ref(torch.tensor(bra, device="cuda")), sec.from_ref(torch.tensor(ket, device="cuda")),
                         pairs=all_pairs(norb))
    ref = O.j_spin_heis(norb, bra, ket)
    assert np.abs(assemble_heisenberg(raw, norb) - ref).max() < 1e-11 * np.abs(ref).max()
    full = LZ.ground_state(sec, mode="f64", steps=300, rule=LZ.ResidualRule(1e-11, 10))
    gs = LZ.ground_state(sec, mode="mixed", steps=150, reorth="none", refine_steps=150,
                         rule=LZ.EnergyRule(1e-9, min_steps=20))
    assert abs(gs.e0 - full.e0) < 1e-9, (gs.e0, full.e0)
    bonds = [(i + 1, j + 1) for i in range(norb) for j in range(norb) if i != j and J[i, j] != 0.0]
    r2, _ = sec.rdm_raw(gs.psi, pairs=bonds)
    e_bonds = sum(J[j - 1, i - 1] * (q[1] - q[0]) for (i, j), q in zip(bonds, r2))
    assert abs(gs.e0 - e_bonds) < 1e-8, (gs.e0, e_bonds)


def test_self_energy_array_matches_per_frequency(edlib):
    """GreenFunction.self_energy on a frequency array (gf_matrix + batched
    pseudo-inverses) equals the reference's per-frequency evaluation, in the
    reference's [j][i][k] layout, to 1e-10 relative; gf_matrix equals the
    Pole objects' retarded values."""
    from pyhub_gb300.solver import FermiHubbard
    norb = 6
    t = O.ring(norb)
    t[0, 3] = t[3, 0] = -0.3
    fh = FermiHubbard(norb, 3, 3, t, 3.0)
    fh.kernel(max_lcz=300, acc_lcz=1e-13, compute_rq=False)
    fh.spgf(nsteps=200)
    w = np.linspace(-6, 6, 41)
    G = fh.gf_matrix(w, eta=0.1)
    for s in ("up", "down"):
        for i in range(norb):
            for j in range(norb):
                ref = fh.gf[s][i, j].retarded(w, eta=0.1)
                assert np.abs(G[s][:, i, j].cpu().numpy() - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())
    S = fh.self_energy(w, eta=0.1)
    for k in (0, 17, 40):
        one = fh.self_energy(w[k], eta=0.1)
        for s in ("up", "down"):
            got = S[s][:, :, k].T
            assert np.abs(got - one[s]).max() <= 1e-10 * max(1.0, np.abs(one[s]).max()), (s, k)


@pytest.mark.parametrize("nu,nd", [(3, 3), (3, 2)])
def test_self_energy_matches_reference_formula(edlib, nu, nd):
    """Sigma(w) and G(w) against the oracle's restatement of the reference's
    self_energy (reduced_quantities.py:134-161) on exact SPGF_ED poles (full ED
    of the N+-1 sectors): G to 1e-9, Sigma to 1e-7 of its largest entry (the
    pseudo-inverses amplify the pole error)."""
    from pyhub_gb300.solver import FermiHubbard
    norb = 6
    t = O.ring(norb)
    t[0, 3] = t[3, 0] = -0.3
    U = 3.0
    fh = FermiHubbard(norb, nu, nd, t, U)
    fh.kernel(max_lcz=300, acc_lcz=1e-13, compute_rq=False)
    fh.spgf(nsteps=400)
    osec = O.Sector(norb, nu, nd)
    H = O.dense_h(lambda v: O.hprod_hubbard(osec, t, U, v, fast=True), osec.dim)
    e, v = np.linalg.eigh(H)
    sp = O.spgf_ed(osec, t, U, [v[:, 0]], norb)
    ek, Vk = np.linalg.eigh(t)
    w = np.array([-3.1, -0.7, 0.2, 1.9, 4.4])
    eta = 0.1
    G = fh.gf_matrix(w, eta=eta, raw=True)
    S = fh.self_energy(w, eta=eta)
    for k, wk in enumerate(w):
        ref = O.self_energy_ref(Vk, ek, e[:1], [1.0], sp, wk, eta, nu == nd)
        for s in ("up", "down"):
            src = "up" if nu == nd else s
            Gr = sum(np.einsum("ik,jk,k->ij", sp[f"Q_{p}_{src}"][:, :, 0], sp[f"Q_{p}_{src}"][:, :, 0],
                               1.0 / (wk - (sg * (sp[f"positions_{p}_{src}"] - e[0])) + 1j * eta))
                     for p, sg in (("greater", 1.0), ("lesser", -1.0)))
            assert np.abs(G[s][k].cpu().numpy() - Gr).max() <= 1e-9 * np.abs(Gr).max(), (s, k)
            got = S[s][:, :, k].T
            assert np.abs(got - ref[s]).max() <= 1e-7 * np.abs(ref[s]).max(), (s, k, np.abs(got - ref[s]).max())
    # the quasi-particle weight at the chemical potential: mu from the lowest N+-1 energies that the
    # start vectors reach (poles of nonzero weight), as ip and ae take them
    def lowest(part):
        w = np.sum(sp[f"Q_{part}_up"][:, :, 0] ** 2, axis=0)
        return float(np.min(sp[f"positions_{part}_up"][w > 1e-12]))
    mu = 0.5 * ((lowest("greater") - e[0]) + (e[0] - lowest("lesser")))
    assert abs(fh.mu["up"] - mu) < 1e-8
    # 1 - Re Sigma'(mu) by the central difference, then its pseudo-inverse (compared where it is
    # well conditioned: the pseudo-inverse amplifies differences by the condition number)
    dx = 1.e-6
    d_ref = np.identity(norb) - np.real(
        (O.self_energy_ref(Vk, ek, e[:1], [1.0], sp, mu + dx, 1e-4, nu == nd)["up"]
         - O.self_energy_ref(Vk, ek, e[:1], [1.0], sp, mu - dx, 1e-4, nu == nd)["up"]) / (2 * dx))
    so = fh.self_energy(np.array([fh.mu["up"] - dx, fh.mu["up"] + dx]), eta=1e-4)["up"]
    d_got = np.identity(norb) - np.real((so[:, :, 1] - so[:, :, 0]).T / (2 * dx))
    assert np.abs(d_got - d_ref).max() <= 1e-4 * np.abs(d_ref).max(), np.abs(d_got - d_ref).max()
    z_ref = O.qpw_ref(Vk, ek, e[:1], [1.0], sp, mu, nu == nd, norb)
    assert np.allclose(z_ref, np.linalg.pinv(d_ref))
    if np.linalg.cond(d_ref) < 1e6:
        z = fh.qpw
        assert np.abs(z - z_ref).max() <= 1e-3 * max(1.0, np.abs(z_ref).max()), np.abs(z - z_ref).max()
    assert fh.galitskii_migdal is None


def test_lanczos_vectors_and_operator_exponential(edlib):
    """lcz_vectors (kept on request by an FP64 solve): orthonormal, V^T H V is
    the tridiagonal of alpha/beta, and V times its lowest eigenvector is psi0.
    opeexp: exp(O) psi by the Taylor series equals expm of the operator's
    matrix applied to psi."""
    import scipy.linalg as sl
    from pyhub_gb300.core.basis import Basis
    from pyhub_gb300.solver import FermiHubbard
    from pyhub_gb300.tools import operators as OP
    t = O.ring(8)
    fh = FermiHubbard(8, 4, 4, t, 4.0)
    fh.kernel(max_lcz=200, acc_lcz=1e-8, compute_rq=False, dtype="f64", reorth="full", store_lanczos_vectors=True)
    V = fh.lcz_vectors
    k = V.shape[1]
    assert k == fh.nb_lcz
    assert np.abs(V.T @ V - np.eye(k)).max() < 1e-10
    osec = O.Sector(8, 4, 4)
    HV = np.stack([O.hprod_hubbard(osec, t, 4.0, V[:, j], fast=True) for j in range(k)], axis=1)
    lcz = fh.lcz_results
    T = np.diag(lcz["alpha"][:k]) + np.diag(lcz["beta"][:k - 1], 1) + np.diag(lcz["beta"][:k - 1], -1)
    assert np.abs(V.T @ HV - T).max() < 1e-9
    e, y = np.linalg.eigh(T)
    assert abs(abs((V @ y[:, 0]) @ fh.psi0) - 1.0) < 1e-8
    fh2 = FermiHubbard(8, 4, 4, t, 4.0)
    fh2.kernel(max_lcz=200, compute_rq=False)
    with pytest.raises(KeyError):
        fh2.lcz_vectors
    op = 0.3 * (OP.c_dagger_c((0, 'u'), (1, 'u')) + OP.c_dagger_c((1, 'u'), (0, 'u'))) + 0.2 * OP.n((2, 'd'))
    op.set_basis(Basis(4, hilbert=(2, 2)))
    psi = np.random.default_rng(2).normal(size=op.nstates)
    M = op.to_matrix
    got = OP.opeexp(op, psi, ftol=1e-14)
    np.testing.assert_allclose(got, sl.expm(M.T) @ psi, rtol=0, atol=1e-10)


def test_ring_energy_approaches_bethe_ansatz(edlib):
    """Half-filled Hubbard rings (U = 4, closed shells L = 4n + 2) against the
    thermodynamic energy per site that the reference's bethe_anzatz.E_bessel(4)
    returns (golden value from the reference's own Python): the finite-size
    error shrinks from L = 10 to L = 14, and the 1/L^2 extrapolation of the two
    lands within 2e-3 of it (a loose physics pin, as the reference's examples
    use it)."""
    import os
    from pyhub_gb300.solver import FermiHubbard
    eb = float(np.load(os.path.join(os.path.dirname(__file__), "golden", "pole_golden.npz"))["e_bessel_U4"])
    e = {}
    for L in (10, 14):
        fh = FermiHubbard(L, L // 2, L // 2, O.ring(L), 4.0)
        fh.kernel(max_lcz=300, acc_lcz=1e-10, compute_rq=False)
        e[L] = fh.e0 / L
    assert abs(e[10] - (-0.5834322635772545)) < 1e-9      # the oracle's Lanczos on the same ring
    assert abs(e[14] - eb) < abs(e[10] - eb) < 0.011
    e_inf = (14 ** 2 * e[14] - 10 ** 2 * e[10]) / (14 ** 2 - 10 ** 2)
    assert abs(e_inf - eb) < 2e-3, (e, e_inf, eb)


@pytest.mark.parametrize("case", [(6, 3, 3), (6, 2, 4)])
def test_composite_entry_points(edlib, case):
    """ed_rdm1 equals the Python assembly of the same ed_rdm sums bit for bit;
    ed_hf_grad equals the Hellmann-Feynman gradient of core.gradients to
    1e-12; m calls of ed_lanczos_step give lanczos_full's alpha/beta bit for
    bit (same kernels, same order)."""
    import torch
    from pyhub_gb300.core import gradients as GRD
    from pyhub_gb300.core import lanczos as LZ
    from pyhub_gb300.core.reduced_quantities import (all_pairs, assemble_heisenberg, assemble_hubbard,
                                                     lower_pairs, scatter_pairs)
    norb, nu, nd = case
    t, U, rng = _state(norb, nu, nd, 3 * norb + nu)
    sec = edlib.Sector(norb, nu, nd, edlib.ED_HUBBARD, t=t, U=U)
    osec = O.Sector(norb, nu, nd)
    psi = rng.standard_normal(osec.dim)
    psi /= np.linalg.norm(psi)
    x = sec.from_ref(torch.tensor(psi, device="cuda"))
    gamma, docc, sisj = sec.rdm1(x)
    pairs = lower_pairs(norb)
    raw, _ = sec.rdm_raw(x, pairs=pairs, flags=2 | (1 if nu != nd else 0))
    gu, gd, ni, sm = assemble_hubbard(scatter_pairs(raw, pairs, norb), norb, nu, nd)
    assert np.array_equal(gamma[0], gu) and np.array_equal(gamma[1], gd)
    assert np.array_equal(docc, ni) and np.array_equal(sisj, sm)
    # gradient: bonds of t, both spins summed
    bonds = [(i, j) for i in range(norb) for j in range(i + 1, norb) if abs(t[i, j]) > 0.3]
    params = GRD.HubbardParams(norb, bonds)
    raw2, _ = sec.rdm_raw(x, pairs=params.pairs(), flags=1)
    g_ref = params.contract(raw2)
    g_t, g_u, g_e = sec.hf_grad(x, [(i + 1, j + 1) for i, j in bonds])
    nb = len(bonds)
    np.testing.assert_allclose(g_t, g_ref[:nb], rtol=0, atol=1e-12)
    np.testing.assert_allclose(g_u, g_ref[nb:nb + norb], rtol=0, atol=1e-12)
    np.testing.assert_allclose(g_e, g_ref[nb + norb:], rtol=0, atol=1e-12)
    # Heisenberg: sisj only
    hs = edlib.Sector(norb, norb // 2, 0, edlib.ED_HEISENBERG, J=O.ring(norb, 1.0))
    y = torch.tensor(rng.standard_normal(hs.dim), device="cuda")
    g0, d0, s0 = hs.rdm1(y)
    rawh, _ = hs.rdm_raw(y, pairs=all_pairs(norb))
    assert g0 is None and d0 is None and np.array_equal(s0, assemble_heisenberg(rawh, norb))
    # Lanczos steps through the C ABI against lanczos_full
    m = 30
    v0 = LZ.start_vector(sec, 4)
    ref = LZ.lanczos_full(sec, v0, m, torch.float64, rule=None, want_vector=False)
    V = torch.zeros((m + 1, sec.n), dtype=torch.float64, device="cuda")
    V[0].copy_(v0)
    w = torch.zeros(sec.n, dtype=torch.float64, device="cuda")
    sc = torch.zeros((sec.lanczos_step_scratch_bytes(m) + 7) // 8, dtype=torch.float64, device="cuda")
    n0 = torch.zeros(2, dtype=torch.float64, device="cuda")
    buf = torch.empty(edlib.scratch_bytes(sec.n, 2) // 8 + 1, dtype=torch.float64, device="cuda")
    edlib.multidot(V, 1, V[0], n0, buf)
    state = torch.zeros(edlib.lanczos_state_doubles(m), dtype=torch.float64, device="cuda")
    state[2] = 1.0 / float(n0[0].item()) ** 0.5
    ab = torch.zeros((2, m), dtype=torch.float64, device="cuda")
    for k in range(m):
        sec.lanczos_step(V, k, m, w, state, ab[0], ab[1], sc)
    torch.cuda.synchronize()
    a = ab[0].cpu().numpy()
    b = ab[1].cpu().numpy()
    assert np.array_equal(a, np.asarray(ref.alpha)[:m]), np.abs(a - np.asarray(ref.alpha)[:m]).max()
    assert np.array_equal(b[:m - 1], np.asarray(ref.beta)[:m - 1])
