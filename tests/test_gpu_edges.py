"""Edge cases of the sector machinery on the GPU: one-state sectors (empty,
full and one-site lattices), and a batch that mixes a one-state instance with
ordinary ones.  Tolerances: H*v and RDMs 1e-14 relative against the oracle;
batched alpha/beta 1e-9 against the per-instance three-term Lanczos."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

TINY = [(1, 0, 0), (1, 1, 0), (1, 1, 1), (3, 3, 3), (6, 6, 0), (5, 0, 5), (4, 4, 1), (4, 0, 4)]


def _tu(norb, seed):
    rng = np.random.default_rng(seed)
    t = rng.standard_normal((norb, norb))
    return 0.5 * (t + t.T), rng.uniform(1, 4, norb)


@pytest.mark.parametrize("case", TINY)
def test_tiny_sector_hv_and_rdm(edlib, case):
    import torch
    norb, nu, nd = case
    t, U = _tu(norb, sum(case))
    sec = edlib.Sector(norb, nu, nd, edlib.ED_HUBBARD, t=t, U=U)
    osec = O.Sector(norb, nu, nd)
    assert sec.dim == osec.dim
    x = np.random.default_rng(1).standard_normal(osec.dim)
    ref = O.hprod_hubbard(osec, t, U, x)
    for dt, tol in ((torch.float64, 1e-14), (torch.float32, 1e-6)):
        xd = sec.from_ref(torch.tensor(x, dtype=dt, device="cuda"))
        yd = torch.zeros_like(xd)
        sec.hv(xd, yd)
        y = sec.to_ref(yd).double().cpu().numpy()
        assert np.linalg.norm(y - ref) <= tol * max(1.0, np.linalg.norm(ref)), (case, dt)
    pairs = [(J, K) for J in range(1, norb + 1) for K in range(1, norb + 1)]
    raw, _ = sec.rdm_raw(sec.from_ref(torch.tensor(x, device="cuda")), pairs=pairs)
    q = raw.reshape(norb, norb, 6)
    oref = O.one_rdm(osec, x, x)
    for J in range(norb):
        # occupations of the one-state sector: n_up = x^2 [J occupied]
        assert abs(q[J, J, 0] - oref["up"][J][J]) <= 1e-12 * max(1.0, float(x @ x))


def test_tiny_sector_api_ground_state(edlib):
    """The API on a one-state sector: E0 is the diagonal element."""
    from pyhub_gb300.solver import FermiHubbard
    t, U = _tu(4, 3)
    fh = FermiHubbard(4, 4, 1, t, U)
    fh.kernel(max_lcz=20, acc_lcz=1e-12)
    osec = O.Sector(4, 4, 1)
    H = O.dense_h(lambda v: O.hprod_hubbard(osec, t, U, v), osec.dim)
    assert abs(fh.e0 - np.linalg.eigvalsh(H)[0]) < 1e-12


def test_batch_with_one_state_instance(edlib):
    import torch
    from pyhub_gb300.core import greens_batched as GB
    t, U = _tu(6, 9)
    secs = [edlib.Sector(6, 3, 2, edlib.ED_HUBBARD, t=t, U=U), edlib.Sector(6, 6, 0, edlib.ED_HUBBARD, t=t, U=U),
            edlib.Sector(6, 2, 4, edlib.ED_HUBBARD, t=t, U=U)]
    bl = GB.BatchedLanczos(secs, 12, dtype=torch.float64)
    rng = np.random.default_rng(2)
    for i, s in enumerate(secs):
        bl.start(i).copy_(s.from_ref(torch.tensor(rng.standard_normal(s.dim), device="cuda")))
    starts = [bl.start(i).clone() for i in range(3)]
    bl.run()
    torch.cuda.synchronize()
    A, B = bl.alpha.cpu().numpy(), bl.beta.cpu().numpy()
    # the one-state instance: alpha_0 is its energy, the next beta vanishes
    osec = O.Sector(6, 6, 0)
    e = O.hprod_hubbard(osec, t, U, np.ones(1))[0]
    assert abs(A[1, 0] - e) < 1e-12 and B[1, 1] < 1e-12
    for i in (0, 2):
        a, b = GB.plain_coefficients(secs[i], starts[i], 12)
        n = np.count_nonzero(b[1:] > 1e-8)
        assert np.allclose(A[i, :n], a[:n], rtol=1e-9, atol=1e-9)
        assert np.allclose(B[i, :n + 1], b[:n + 1], rtol=1e-9, atol=1e-9)


@pytest.mark.parametrize("dt", ["f64", "f32"])
def test_full_lanczos_breakdown_on_small_sector(edlib, dt):
    """A 24-state sector run for 40 full-reorthogonalisation steps.  FP64: the
    Krylov space is exhausted and the device stop code ends the run at <= 24
    steps.  FP32: the next vector is rounding noise (~1e-7 ||H||, above the
    breakdown threshold), so the run goes on with noise directions, as the
    reference's recurrence would.  Either way the lowest Ritz value is E0 of
    the dense matrix (1e-10 FP64, 1e-5 FP32) and the Ritz vector is finite and
    normalised."""
    import torch
    from pyhub_gb300.core import lanczos as LZ
    t, U = _tu(4, 11)
    sec = edlib.Sector(4, 2, 1, edlib.ED_HUBBARD, t=t, U=U)
    assert sec.dim == 24
    td = torch.float64 if dt == "f64" else torch.float32
    r = LZ.lanczos_full(sec, LZ.start_vector(sec, 2, dtype=td), 40, td)
    osec = O.Sector(4, 2, 1)
    e = np.linalg.eigvalsh(O.dense_h(lambda v: O.hprod_hubbard(osec, t, U, v), osec.dim))[0]
    if dt == "f64":
        assert r.breakdown and r.steps <= 24
    assert abs(r.ritz[0] - e) < (1e-10 if dt == "f64" else 1e-5)
    assert bool(torch.isfinite(r.psi).all())
    assert abs(float(torch.linalg.vector_norm(r.psi)) - 1.0) < 1e-12
