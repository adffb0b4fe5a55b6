"""GPU parity of the FP32 Hubbard H*v on 16-site sectors (the 4x4 lattice's
site count) against the CPU oracle: 8 particles of one spin with every other
count of the other, so that both the row pass (up hops, one row of 12,870 up
strings staged in shared memory) and the slab pass (down hops over 12,870
rows) run at the benchmark's string-table sizes.

Tolerances:
  integer-valued t, U and x: bit-exact;
  real-valued: per element |y - y_ref| <= 64 eps32 (|d_i||x_i| + h_max |t|_max |x|_max),
      y_ref the FP64 oracle product of the same FP32-rounded x, d_i the diagonal
      and h_max the most hops a basis state has (8*8 up + 8*8 down).
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

EPS32 = float(np.finfo(np.float32).eps)

def _params(seed, integer, sym, lattice=False):
    rng = np.random.default_rng(seed)
    if lattice:
        t = O.square_pbc(4, 4, -1.0) + np.diag(rng.integers(-2, 3, 16).astype(np.float64))
        U = 4.0
    elif integer:
        t = rng.integers(-3, 4, size=(16, 16)).astype(np.float64)
        U = float(rng.integers(0, 9))
    else:
        t = rng.standard_normal((16, 16))
        U = float(rng.uniform(0.0, 8.0))
    if sym:
        t = np.triu(t) + np.triu(t, 1).T
    # one amplitude below the single-precision 1.E-14 threshold, one exactly zero
    t[2, 11] = 1e-16
    t[5, 6] = 0.0
    return t, U, rng


def _hv32(edlib, sec, x, ld=None):
    import torch
    xr = torch.tensor(x, dtype=torch.float32, device="cuda")
    if ld is None:
        y = torch.full_like(xr, float("nan"))
        sec.hv(xr, y, ld=sec.nsup)
        torch.cuda.synchronize()
        return y.double().cpu().numpy()
    xi = sec.from_ref(xr)
    yi = torch.zeros_like(xi)
    sec.hv(xi, yi)
    torch.cuda.synchronize()
    return sec.to_ref(yi).double().cpu().numpy()


def _diag(osec, t, U):
    """Diagonal of H: the oracle product on unit vectors would be dim calls; the
    diagonal is the one-body energies plus U times the double occupancy."""
    ups, dns = osec.bup, osec.bdn
    tf = t.reshape(-1)
    eps = np.array([tf[(J - 1) * 16 + (J - 1)] for J in range(1, 17)])
    eps[np.abs(eps) < float(np.float32(1e-14))] = 0.0
    bits = lambda s: np.array([(int(s) >> (16 - J)) & 1 for J in range(1, 17)])
    bu = np.array([bits(s) for s in ups])
    bd = np.array([bits(s) for s in dns])
    eu, ed = bu @ eps, bd @ eps
    both = bd @ bu.T                      # [down, up] doubly occupied sites
    return (ed[:, None] + eu[None, :] + U * both).reshape(-1)


CASES = [(8, 0), (8, 1), (8, 2), (8, 15), (8, 16), (0, 8), (1, 8), (2, 8), (15, 8), (16, 8)]


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("kind", ["integer", "real", "real_nonsym", "lattice"])
def test_hubbard_16_sites_f32_matches_oracle(edlib, case, kind):
    nup, ndn = case
    integer = kind in ("integer", "lattice")
    t, U, rng = _params(100 + 17 * nup + ndn, integer, sym=kind != "real_nonsym", lattice=kind == "lattice")
    osec = O.Sector(16, nup, ndn)
    sec = edlib.Sector(16, nup, ndn, edlib.ED_HUBBARD, t=t, U=np.full(16, U))
    if integer:
        x = rng.integers(-4, 5, size=osec.dim).astype(np.float64)
    else:
        x = rng.standard_normal(osec.dim).astype(np.float32).astype(np.float64)
    yref = O.hprod_hubbard(osec, t, np.full(16, U), x, fast=True)
    for ld in (None, "padded"):
        y = _hv32(edlib, sec, x, None if ld is None else sec.ld)
        if integer:
            assert np.array_equal(y, yref)
        else:
            d = _diag(osec, t, U)
            bound = 64 * EPS32 * (np.abs(d) * np.abs(x) + 128 * np.abs(t).max() * np.abs(x).max())
            assert np.all(np.abs(y - yref) <= bound)
            assert np.linalg.norm(y - yref) <= 1e-5 * np.linalg.norm(yref)


def test_hubbard_16_sites_7_8_integer_exact(edlib):
    """N_up = 7, N_down = 8 (D = 1.47e8, both passes at full string-table
    sizes, N_up != N_down): bit-exact on integers."""
    t, U, rng = _params(5, integer=True, sym=False)
    osec = O.Sector(16, 7, 8)
    sec = edlib.Sector(16, 7, 8, edlib.ED_HUBBARD, t=t, U=np.full(16, U))
    x = rng.integers(-4, 5, size=osec.dim).astype(np.float64)
    yref = O.hprod_hubbard(osec, t, np.full(16, U), x, fast=True)
    assert np.array_equal(_hv32(edlib, sec, x), yref)
