"""GPU parity of the sector H*v products against the CPU oracle.

Tolerances:
  FP64, real-valued t/U/x: ||y - y_ref|| <= 1e-14 ||y_ref|| and, per element,
      |y - y_ref| <= 64 eps64 (|H||x|)_i;
  FP64 and FP32, integer-valued t, U and x: bit-exact;
  FP32 storage and accumulation: per element |y - y_ref| <= 64 eps32 (|H||x|)_i
      with y_ref the FP64 product of the same FP32-rounded x.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

HUB_CASES = [(2, 1, 1), (4, 2, 2), (5, 2, 3), (6, 3, 3), (6, 2, 4), (7, 3, 2), (8, 4, 4), (8, 1, 7),
             (9, 4, 5), (10, 5, 5), (10, 0, 3), (6, 3, 0), (4, 4, 4), (12, 6, 6), (12, 5, 6)]
EPS64 = np.finfo(np.float64).eps
EPS32 = float(np.finfo(np.float32).eps)


def _params(norb, seed, integer=False, sym=True):
    rng = np.random.default_rng(seed)
    if integer:
        t = rng.integers(-3, 4, size=(norb, norb)).astype(np.float64)
        U = rng.integers(0, 9, size=norb).astype(np.float64)
    else:
        t = rng.standard_normal((norb, norb))
        U = rng.uniform(0.0, 8.0, norb)
    if sym:
        t = np.triu(t) + np.triu(t, 1).T
    return t, U, rng


def _abs_bound(osec, t, U, x):
    """(|H| |x|)_i from the dense oracle matrix (small sectors only)."""
    H = O.dense_h(lambda v: O.hprod_hubbard(osec, t, U, v, fast=True), osec.dim)
    return np.abs(H) @ np.abs(x)


def _run(edlib, sec, x_np, dtype, ld=None):
    import torch
    if ld is None or ld == sec.nsup:
        xd = torch.tensor(x_np, dtype=dtype, device="cuda")
        yd = torch.full_like(xd, float("nan"))
        sec.hv(xd, yd, ld=sec.nsup)
        torch.cuda.synchronize()
        return yd.double().cpu().numpy()
    xr = torch.tensor(x_np, dtype=dtype, device="cuda")
    xi = sec.from_ref(xr)
    yi = torch.zeros_like(xi)
    sec.hv(xi, yi)
    torch.cuda.synchronize()
    return sec.to_ref(yi).double().cpu().numpy()


@pytest.mark.parametrize("case", HUB_CASES)
@pytest.mark.parametrize("layout", ["ref", "padded"])
def test_hubbard_f64_matches_oracle(edlib, case, layout):
    import torch
    norb, nu, nd = case
    t, U, rng = _params(norb, 1000 * norb + 10 * nu + nd)
    osec = O.Sector(norb, nu, nd)
    sec = edlib.Sector(norb, nu, nd, edlib.ED_HUBBARD, t=t, U=U)
    x = rng.standard_normal(osec.dim)
    yref = O.hprod_hubbard(osec, t, U, x, fast=osec.dim > 3000)
    y = _run(edlib, sec, x, torch.float64, None if layout == "ref" else sec.ld)
    assert np.linalg.norm(y - yref) <= 1e-14 * np.linalg.norm(yref) + 1e-300
    if osec.dim <= 2000:
        bound = 64 * EPS64 * _abs_bound(osec, t, U, x)
        assert np.all(np.abs(y - yref) <= bound + 1e-300)


@pytest.mark.parametrize("case", HUB_CASES)
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_hubbard_integer_exact(edlib, case, dtype):
    import torch
    norb, nu, nd = case
    t, U, rng = _params(norb, 7 + norb * 31 + nu, integer=True, sym=False)
    osec = O.Sector(norb, nu, nd)
    sec = edlib.Sector(norb, nu, nd, edlib.ED_HUBBARD, t=t, U=U)
    x = rng.integers(-8, 9, size=osec.dim).astype(np.float64)
    yref = O.hprod_hubbard(osec, t, U, x, fast=osec.dim > 3000)
    td = torch.float64 if dtype == "f64" else torch.float32
    for layout in (None, sec.ld):
        y = _run(edlib, sec, x, td, layout)
        assert np.array_equal(y, yref), f"max diff {np.abs(y - yref).max()}"


@pytest.mark.parametrize("case", [(4, 2, 2), (6, 3, 3), (6, 2, 4), (8, 4, 4), (9, 4, 5)])
def test_hubbard_f32_within_bound(edlib, case):
    import torch
    norb, nu, nd = case
    t, U, rng = _params(norb, 99 + norb)
    osec = O.Sector(norb, nu, nd)
    sec = edlib.Sector(norb, nu, nd, edlib.ED_HUBBARD, t=t, U=U)
    x = rng.standard_normal(osec.dim).astype(np.float32).astype(np.float64)
    yref = O.hprod_hubbard(osec, t, U, x, fast=True)
    bound = 64 * EPS32 * _abs_bound(osec, t, U, x)
    for layout in (None, sec.ld):
        y = _run(edlib, sec, x, torch.float32, layout)
        assert np.all(np.abs(y - yref) <= bound + 1e-30)


@pytest.mark.parametrize("case", [(4, 2, 2), (8, 4, 4), (9, 4, 5), (12, 6, 6), (12, 5, 7)])
def test_hubbard_f32_single_magnitude_hopping(edlib, case):
    """Hopping of one magnitude with both signs (the 2-byte-slot row pass),
    with per-site U and on-site energies: bit-exact for integer x; for an
    FP32-rounded real x, against the oracle's FP64 product, per element within
    64 eps32 (|H||x|)_i where the dense |H| is available, else within 64 eps32
    in norm."""
    import torch
    norb, nu, nd = case
    rng = np.random.default_rng(3 * norb + nu)
    mask = rng.random((norb, norb)) < 0.45
    t = np.where(mask, np.where(rng.random((norb, norb)) < 0.5, -1.0, 1.0), 0.0)
    t = np.triu(t, 1) + np.triu(t, 1).T
    t[np.diag_indices(norb)] = rng.integers(-2, 3, norb)
    U = rng.integers(0, 9, norb).astype(np.float64)
    osec = O.Sector(norb, nu, nd)
    sec = edlib.Sector(norb, nu, nd, edlib.ED_HUBBARD, t=t, U=U)
    xi = rng.integers(-8, 9, size=osec.dim).astype(np.float64)
    yi = O.hprod_hubbard(osec, t, U, xi, fast=True)
    for layout in (None, sec.ld):
        assert np.array_equal(_run(edlib, sec, xi, torch.float32, layout), yi)
    x = rng.standard_normal(osec.dim).astype(np.float32).astype(np.float64)
    yref = O.hprod_hubbard(osec, t, U, x, fast=True)
    y = _run(edlib, sec, x, torch.float32, sec.ld)
    if osec.dim <= 5000:
        assert np.all(np.abs(y - yref) <= 64 * EPS32 * _abs_bound(osec, t, U, x) + 1e-30)
    else:
        # larger sectors: the dense |H| is out of reach; FP32 accumulation of ~20 terms per element
        assert np.linalg.norm(y - yref) <= 64 * EPS32 * np.linalg.norm(yref)


def test_hubbard_fused_dots(edlib):
    import torch
    norb, nu, nd = 10, 5, 4
    t, U, rng = _params(norb, 5)
    osec = O.Sector(norb, nu, nd)
    sec = edlib.Sector(norb, nu, nd, edlib.ED_HUBBARD, t=t, U=U)
    x = rng.standard_normal(osec.dim)
    yref = 0.5 * O.hprod_hubbard(osec, t, U, x, fast=True)
    scratch = torch.empty(edlib.scratch_bytes(sec.n, 1) // 8 + 1, dtype=torch.float64, device="cuda")
    dots = torch.zeros(2, dtype=torch.float64, device="cuda")
    for dt, tol in ((torch.float64, 1e-13), (torch.float32, 1e-5)):
        xi = sec.from_ref(torch.tensor(x, dtype=dt, device="cuda"))
        yi = torch.zeros_like(xi)
        sec.hv(xi, yi, scale=0.5, dots=dots, scratch=scratch)
        d = dots.cpu().numpy()
        assert abs(d[0] - x @ yref) <= tol * abs(x @ yref)
        assert abs(d[1] - yref @ yref) <= tol * (yref @ yref)


@pytest.mark.parametrize("norb", [2, 4, 6, 8, 10, 12])
def test_heisenberg_f64_matches_oracle(edlib, norb):
    import torch
    rng = np.random.default_rng(norb)
    J = rng.standard_normal((norb, norb))
    J = np.triu(J) + np.triu(J, 1).T
    sec = edlib.Sector(norb, norb // 2, 0, edlib.ED_HEISENBERG, J=J)
    x = rng.standard_normal(sec.dim)
    yref = O.hprod_heis(norb, J, x)
    xd = sec.from_ref(torch.tensor(x, device="cuda"))
    yd = torch.zeros_like(xd)
    sec.hv(xd, yd)
    y = sec.to_ref(yd).cpu().numpy()
    assert np.linalg.norm(y - yref) <= 1e-14 * np.linalg.norm(yref)


@pytest.mark.parametrize("norb", [1, 3, 5, 7, 9, 13])
def test_heisenberg_odd_sites_matches_oracle(edlib, norb):
    """Odd site counts: halves of unequal size (nA = norb//2) and N = norb//2 up spins."""
    import torch
    rng = np.random.default_rng(100 + norb)
    J = rng.standard_normal((norb, norb))
    J = np.triu(J) + np.triu(J, 1).T
    sec = edlib.Sector(norb, norb // 2, 0, edlib.ED_HEISENBERG, J=J)
    x = rng.standard_normal(sec.dim)
    yref = O.hprod_heis(norb, J, x)
    xd = sec.from_ref(torch.tensor(x, device="cuda"))
    yd = torch.zeros_like(xd)
    sec.hv(xd, yd)
    y = sec.to_ref(yd).cpu().numpy()
    assert np.linalg.norm(y - yref) <= 1e-14 * np.linalg.norm(yref)


@pytest.mark.parametrize("shape", [(4, 4), (4, 6)])
def test_heisenberg_lattice_with_fused_dots(edlib, shape):
    """Periodic lattices (16 and 24 sites, dims 12,870 and 2,704,156): FP64
    product within 1e-14 of the oracle, fused <x,y> and <y,y> within 1e-12;
    FP32 within 2e-6 relative."""
    import torch
    lx, ly = shape
    norb = lx * ly
    J = O.square_pbc(lx, ly, 1.0)
    rng = np.random.default_rng(norb)
    sec = edlib.Sector(norb, norb // 2, 0, edlib.ED_HEISENBERG, J=J)
    x = rng.standard_normal(sec.dim)
    yref = O.hprod_heis(norb, J, x, fast=True)
    xd = sec.from_ref(torch.tensor(x, device="cuda"))
    yd = torch.zeros_like(xd)
    dots = torch.zeros(2, dtype=torch.float64, device="cuda")
    scratch = torch.empty(edlib.scratch_bytes(sec.n, 1) // 8 + 1, dtype=torch.float64, device="cuda")
    sec.hv(xd, yd, dots=dots, scratch=scratch)
    y = sec.to_ref(yd).cpu().numpy()
    assert np.linalg.norm(y - yref) <= 1e-14 * np.linalg.norm(yref)
    d = dots.cpu().numpy()
    assert abs(d[0] - x @ yref) <= 1e-12 * np.linalg.norm(x) * np.linalg.norm(yref)
    assert abs(d[1] - yref @ yref) <= 1e-12 * (yref @ yref)
    xf = xd.float()
    yf = torch.zeros_like(xf)
    sec.hv(xf, yf)
    y32 = sec.to_ref(yf).double().cpu().numpy()
    assert np.linalg.norm(y32 - yref) <= 2e-6 * np.linalg.norm(yref)


@pytest.mark.parametrize("norb", [4, 8, 12, 14])
def test_heisenberg_integer_exact(edlib, norb):
    import torch
    J = O.ring(norb, 1.0) + 2 * np.diag(np.ones(norb))
    J[0, norb // 2] = J[norb // 2, 0] = 3.0
    rng = np.random.default_rng(3)
    sec = edlib.Sector(norb, norb // 2, 0, edlib.ED_HEISENBERG, J=J)
    x = rng.integers(-8, 9, size=sec.dim).astype(np.float64)
    yref = O.hprod_heis(norb, J, x, fast=True)
    for dt in (torch.float64, torch.float32):
        xd = sec.from_ref(torch.tensor(x, dtype=dt, device="cuda"))
        yd = torch.zeros_like(xd)
        sec.hv(xd, yd)
        y = sec.to_ref(yd).double().cpu().numpy()
        assert np.array_equal(y, yref)


@pytest.mark.parametrize("case", ["4x4", "4x6", "ring13", "ring14_extra"])
def test_heisenberg_four_row_pass_equals_one_row_pass(edlib, monkeypatch, case):
    """FP32: the row pass with four rows of one hole count per CTA and the
    one-row pass (PYHUB_ED_HEIS_ROWS=1) give the same product bit for bit.
    Every case has at most 32 bonds between the halves (the packed path both
    passes need), so the four-row pass runs."""
    import torch
    rng = np.random.default_rng(7)
    if case == "4x4":
        norb, J = 16, O.square_pbc(4, 4, 1.0)
    elif case == "4x6":
        norb, J = 24, O.square_pbc(4, 6, 1.0)
    elif case == "ring13":
        norb = 13
        J = O.ring(13, 1.0) + np.diag(rng.standard_normal(13))
    else:
        norb = 14
        J = O.ring(14, 0.7)
        for _ in range(12):
            i, j = rng.choice(14, size=2, replace=False)
            J[i, j] = J[j, i] = rng.uniform(0.2, 1.5)
    sec = edlib.Sector(norb, norb // 2, 0, edlib.ED_HEISENBERG, J=J)
    xi = sec.from_ref(torch.tensor(rng.standard_normal(sec.dim), dtype=torch.float32, device="cuda"))
    out = []
    for mode in ("0", "1"):
        monkeypatch.setenv("PYHUB_ED_HEIS_ROWS", mode)
        y = torch.zeros_like(xi)
        sec.hv(xi, y, scale=0.75)
        torch.cuda.synchronize()
        out.append(y.cpu().numpy())
    monkeypatch.delenv("PYHUB_ED_HEIS_ROWS")
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("dt", ["f32", "f64"])
def test_multidot_and_update(edlib, dt):
    import torch
    td = torch.float32 if dt == "f32" else torch.float64
    rng = np.random.default_rng(11)
    n, nvec = 100_003, 7
    n_pad = (n + 31) // 32 * 32
    V = torch.zeros((nvec, n_pad), dtype=td, device="cuda")
    Vh = rng.standard_normal((nvec, n)).astype(np.float32 if dt == "f32" else np.float64)
    V[:, :n] = torch.tensor(Vh, device="cuda")
    w = torch.zeros(n_pad, dtype=td, device="cuda")
    wh = rng.standard_normal(n).astype(Vh.dtype)
    w[:n] = torch.tensor(wh, device="cuda")
    scratch = torch.empty(edlib.scratch_bytes(n_pad, nvec) // 8 + 1, dtype=torch.float64, device="cuda")
    out = torch.zeros(2 * nvec, dtype=torch.float64, device="cuda")
    edlib.multidot(V, nvec, w, out, scratch, z=V[2], n=n_pad)
    Vd, wd = Vh.astype(np.float64), wh.astype(np.float64)
    ref = np.concatenate([Vd @ wd, Vd @ Vd[2]])
    tol = 1e-6 if dt == "f32" else 1e-13
    got = out.cpu().numpy()
    assert np.all(np.abs(got - ref) <= tol * np.sqrt((Vd * Vd).sum(1).repeat(1)).max() * np.linalg.norm(wd) * 4)
    coef = rng.standard_normal(nvec)
    cd = torch.tensor(coef, device="cuda")
    o = torch.zeros_like(w)
    nrm = torch.zeros(1, dtype=torch.float64, device="cuda")
    edlib.update(V, nvec, cd, w, o, norm2=nrm, scratch=scratch, n=n_pad)
    refo = wd - coef @ Vd
    oo = o[:n].double().cpu().numpy()
    assert np.abs(oo - refo).max() <= (1e-5 if dt == "f32" else 1e-12) * np.abs(refo).max()
    assert abs(nrm.item() - (oo @ oo)) <= (1e-6 if dt == "f32" else 1e-12) * (oo @ oo)
    # Ritz-vector form: FP64 output from the basis alone
    o64 = torch.zeros(n_pad, dtype=torch.float64, device="cuda")
    edlib.update(V, nvec, cd, None, o64, n=n_pad)
    assert np.abs(o64[:n].cpu().numpy() + coef @ Vd).max() <= 1e-12 * np.abs(coef @ Vd).max()


@pytest.mark.parametrize("mode", ["f64", "mixed"])
def test_lanczos_c1_ring(edlib, mode):
    """L=8 ring, U=4, N_up=N_down=4 (D=4900): E0 against dense diagonalisation."""
    from pyhub_gb300.core import lanczos as LZ
    sec = edlib.Sector(8, 4, 4, edlib.ED_HUBBARD, t=O.ring(8), U=np.full(8, 4.0))
    gs = LZ.ground_state(sec, mode=mode, steps=120, seed=0)
    osec = O.Sector(8, 4, 4)
    H = O.dense_h(lambda v: O.hprod_hubbard(osec, O.ring(8), 4.0, v, fast=True), osec.dim)
    e = np.linalg.eigvalsh(H)
    assert abs(gs.e0 - e[0]) < 1e-10
    # Ritz vector is an eigenvector: residual in FP64
    psi = sec.to_ref(gs.psi).cpu().numpy()
    r = H @ psi - gs.e0 * psi
    assert np.linalg.norm(r) < 1e-6


@pytest.mark.parametrize("dt", ["f32", "f64"])
def test_long_lanczos_stays_bounded(edlib, dt):
    """300 full-reorth steps: stored vectors keep norms of order ||H|| (no
    overflow of the unnormalised basis) and the Gram matrix stays the identity."""
    import torch
    from pyhub_gb300.core import lanczos as LZ
    from pyhub_gb300.tools import lattices as LT
    t = LT.square(3, 3, -1.0)
    sec = edlib.Sector(9, 4, 5, edlib.ED_HUBBARD, t=t, U=np.full(9, 8.0))
    td = torch.float32 if dt == "f32" else torch.float64
    r = LZ.lanczos_full(sec, LZ.start_vector(sec, 0, dtype=td), 300, td, keep_basis=True, want_vector=False)
    assert r.steps == 300 or r.breakdown
    nrm = torch.linalg.vector_norm(r.basis[: r.steps].double(), dim=1).cpu().numpy()
    assert np.all(np.isfinite(nrm)) and nrm.max() < 1e3
    assert r.gram_offdiag < (1e-5 if dt == "f32" else 1e-12)
    osec = O.Sector(9, 4, 5)
    e = O.lanczos_ref(lambda v: O.hprod_hubbard(osec, t, 8.0, v, fast=True),
                      np.random.default_rng(0).uniform(-0.5, 0.5, osec.dim), 600, 1e-12)["eigenvalues"][0]
    assert abs(r.ritz[0] - e) < (1e-5 if dt == "f32" else 1e-10)
    r.release()


@pytest.mark.parametrize("case", [(7, 3, 2), (8, 4, 4), (9, 4, 5), (16, 8, 8)])
def test_padded_and_reference_layouts_bit_identical(edlib, case):
    """FP32 product in the padded layout (16-byte rows: the slab pass loads
    four columns per lane) and in the reference layout (rows of C(n,k) = 2 mod 4
    entries: one column per lane).  Both sum the same terms in the same order,
    so the products agree bit for bit; the fused dots agree to rounding of
    FP32 partial sums grouped differently (4x4 included, D = 165,636,900)."""
    import torch
    norb, nu, nd = case
    if norb == 16:
        t = O.square_pbc(4, 4)
        U = np.full(16, 8.0)
    else:
        t, U, _ = _params(norb, 7 * norb + nu)
    sec = edlib.Sector(norb, nu, nd, edlib.ED_HUBBARD, t=t, U=U)
    assert sec.nsup % 4 != 0
    g = torch.Generator(device="cuda")
    g.manual_seed(11)
    xr = torch.rand(sec.dim, generator=g, device="cuda", dtype=torch.float32) - 0.5
    yr = torch.full_like(xr, float("nan"))
    sc = torch.empty(edlib.scratch_bytes(sec.n, 1) // 8 + 1, dtype=torch.float64, device="cuda")
    d_ref = torch.zeros(2, dtype=torch.float64, device="cuda")
    sec.hv(xr, yr, dots=d_ref, scratch=sc, ld=sec.nsup)          # reference layout
    xi = sec.from_ref(xr)
    yi = torch.zeros_like(xi)
    d_pad = torch.zeros(2, dtype=torch.float64, device="cuda")
    sec.hv(xi, yi, dots=d_pad, scratch=sc)                       # padded layout
    torch.cuda.synchronize()
    assert torch.equal(sec.to_ref(yi), yr)
    a, b = d_ref.cpu().numpy(), d_pad.cpu().numpy()
    assert np.all(np.abs(a - b) <= 1e-5 * max(np.abs(a).max(), 1.0)), (a, b)
    del xr, yr, xi, yi
    torch.cuda.empty_cache()
