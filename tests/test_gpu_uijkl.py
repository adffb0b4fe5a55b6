"""The general two-body interaction U_ijkl (the reference's is_Uloc=3 path,
hprod_hubbard.f90:37,62-86) and the two-body density DBL_OCC
(static_rq.f90:256-306) against the oracle.

Tolerances: H*v FP64 <= 1e-14 relative (norm); bit-exact for integer t, U
and x in FP64 and FP32; DBL_OCC <= 1e-12 of the largest |DBL_OCC| and
bit-exact for integer bra/ket; E0 of FermiHubbard with a U tensor <= 1e-10
against dense diagonalisation of the oracle's matrix."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = [(4, 2, 2), (5, 2, 3), (6, 3, 3), (6, 2, 4), (7, 3, 3), (8, 4, 4)]


def _params(n, seed, integer=False, density=0.3):
    rng = np.random.default_rng(seed)
    if integer:
        t = rng.integers(-2, 3, (n, n)).astype(np.float64)
        Ul = rng.integers(-3, 4, (n,) * 4).astype(np.float64) * (rng.random((n,) * 4) < density)
    else:
        t = rng.standard_normal((n, n))
        Ul = rng.standard_normal((n,) * 4) * (rng.random((n,) * 4) < density)
    t = np.triu(t) + np.triu(t, 1).T
    Ul = Ul + np.einsum("ijkl->jilk", Ul)    # symmetric as the reference requires
    Ul[1, 0] = Ul[0, 1] = 0.0                # (J,K) = (1,2), (2,1) gated off by UPARTIAL, still symmetric
    return t, Ul, rng


def _sector(edlib, n, nu, nd, t, Ul):
    sec = edlib.Sector(n, nu, nd, edlib.ED_HUBBARD, t=t, U=np.zeros(n))
    sec.set_uijkl(Ul)
    return sec


@pytest.mark.parametrize("case", CASES)
def test_uijkl_hv_matches_oracle(edlib, case):
    import torch
    n, nu, nd = case
    t, Ul, rng = _params(n, 10 * n + nu)
    osec = O.Sector(n, nu, nd)
    sec = _sector(edlib, n, nu, nd, t, Ul)
    x = rng.standard_normal(osec.dim)
    yref = O.hprod_hubbard_uijkl(osec, t, Ul, x)
    xd = sec.from_ref(torch.tensor(x, device="cuda"))
    yd = torch.zeros_like(xd)
    sec.hv(xd, yd)
    y = sec.to_ref(yd).cpu().numpy()
    assert np.linalg.norm(y - yref) <= 1e-14 * np.linalg.norm(yref)


@pytest.mark.parametrize("case", CASES)
def test_uijkl_hv_integer_exact(edlib, case):
    import torch
    n, nu, nd = case
    t, Ul, rng = _params(n, 3 * n + nd, integer=True)
    osec = O.Sector(n, nu, nd)
    sec = _sector(edlib, n, nu, nd, t, Ul)
    x = rng.integers(-4, 5, osec.dim).astype(np.float64)
    yref = O.hprod_hubbard_uijkl(osec, t, Ul, x)
    for dt in (torch.float64, torch.float32):
        xd = sec.from_ref(torch.tensor(x, dtype=dt, device="cuda"))
        yd = torch.zeros_like(xd)
        sec.hv(xd, yd)
        assert np.array_equal(sec.to_ref(yd).double().cpu().numpy(), yref), dt


@pytest.mark.parametrize("case", [(4, 2, 2), (5, 2, 3), (6, 3, 2)])
def test_dbl_occ_matches_oracle(edlib, case):
    import torch
    n, nu, nd = case
    rng = np.random.default_rng(n + 7 * nu)
    osec = O.Sector(n, nu, nd)
    sec = edlib.Sector(n, nu, nd, edlib.ED_HUBBARD, t=O.ring(n), U=np.zeros(n))
    quads = [(J, K, M, N) for J in range(1, n + 1) for K in range(1, J + 1)
             for M in range(1, n + 1) for N in range(1, M + 1)]
    for integer in (False, True):
        if integer:
            bra, ket = (rng.integers(-3, 4, osec.dim).astype(np.float64) for _ in range(2))
        else:
            bra, ket = rng.standard_normal(osec.dim), rng.standard_normal(osec.dim)
        ref, ni = O.two_rdm_dbl_occ(osec, bra, ket)
        for dt in ((torch.float64, torch.float32) if integer else (torch.float64,)):
            b = sec.from_ref(torch.tensor(bra, dtype=dt, device="cuda"))
            k = sec.from_ref(torch.tensor(ket, dtype=dt, device="cuda"))
            got, _ = sec.dbl_occ(b, k, quads=quads)
            want = np.array([ref[J - 1, K - 1, M - 1, N - 1] for (J, K, M, N) in quads])
            if integer:
                assert np.array_equal(got, want), dt
            else:
                assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()


@pytest.mark.parametrize("case,max_lcz", [((5, 2, 2), 600), ((6, 3, 3), 300)])
def test_fermi_hubbard_with_u_tensor(edlib, case, max_lcz):
    """FermiHubbard(U=tensor): E0 (exact diagonalisation below max_lcz, Lanczos
    above) against the oracle's dense matrix; two_rdm, ni and the energy
    pieces against the oracle's DBL_OCC of the oracle ground state."""
    from pyhub_gb300.solver import FermiHubbard
    n, nu, nd = case
    t, Ul, _ = _params(n, 77 + n, density=0.2)
    osec = O.Sector(n, nu, nd)
    H = O.dense_h(lambda v: O.hprod_hubbard_uijkl(osec, t, Ul, v), osec.dim)
    e, v = np.linalg.eigh(H)
    assert e[1] - e[0] > 1e-6
    fh = FermiHubbard(n, nu, nd, t, Ul)
    fh.kernel(max_lcz=max_lcz, acc_lcz=1e-12)
    assert abs(fh.e0 - e[0]) < 1e-10
    ref, ni = O.two_rdm_dbl_occ(osec, v[:, 0], v[:, 0])
    assert np.abs(fh.two_rdm - ref).max() < 1e-8
    assert np.abs(fh.ni - ni).max() < 1e-8
    assert abs(fh.e_two_body - (np.einsum("ijkl,ijkl->", ref, Ul) +
                                np.einsum("ij,ij->", fh.spin_cor_matrix, fh.J_matrix))) < 1e-8


def test_u_tensor_must_be_symmetric(edlib):
    from pyhub_gb300.solver import FermiHubbard
    n = 4
    Ul = np.zeros((n,) * 4)
    Ul[0, 1, 2, 3] = 1.0
    fh = FermiHubbard(n, 2, 2, O.ring(n), Ul)
    with pytest.raises(ValueError, match="symmetric"):
        fh.kernel()
