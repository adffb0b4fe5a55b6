"""Parity at the benchmark sizes.

Against the oracle:
* 4x4 Hubbard (t=1, U=8, D=165,636,900): one whole FP64 product against the
  reference loop restated in C (hprod_hubbard.f90:17-118, run on all host
  threads, a few seconds): ||y - y_ref|| <= 1e-14 ||y_ref||, and bit-exact
  (FP64 and FP32) for an integer-valued x.
* 4x8 Heisenberg (J=1, D=601,080,390, past the reference's int32 strings):
  the oracle reads HPROD (hprod_heis.f90:1-61) from the output side on
  ~1e5 seeded sampled rows, with inputs that are a function of the element
  index (oracle.hashvec), compared per row at 64 eps64 (|H||x|)_i and
  bit-exact for integer inputs; J_SPIN (static_rq_heis.f90:58-116) of the
  nearest-neighbour bonds with the bra restricted to the sampled rows, at
  1e-12 of the sum of the terms' magnitudes and bit-exact for integers.
Size-independent properties:
* the same two sectors: with integer-valued inputs every partial sum is an
  exact FP32 number, so the FP32 and FP64 products must be equal bit for bit;
  and <x1, H x2> = <H x1, x2> (H symmetric) in FP64 to 1e-13 relative.
* two 12-site clusters of the batched Green's-function set: the batched
  alpha/beta equal the per-instance three-term Lanczos to 1e-9 (30 steps).
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu
EPS64 = float(np.finfo(np.float64).eps)


def _hash_device(n, seed, kind, dtype):
    """oracle.hashvec of the indices 0..n-1, formed on the device in chunks."""
    import torch
    out = torch.empty(n, dtype=dtype, device="cuda")
    step = 1 << 26
    for a in range(0, n, step):
        i = torch.arange(a, min(n, a + step), dtype=torch.int64, device="cuda")
        h = (i * 2654435761 + seed * 40503) & 0xFFFFFFFF
        v = h.double() / 4294967296.0 - 0.5 if kind == 0 else (h % 7).double() - 3.0
        out[a:a + len(i)] = v.to(dtype)
    return out


def test_hubbard_4x4_fp64_matches_oracle(edlib):
    import torch
    from pyhub_gb300.tools import lattices as LT
    t, U = LT.hubbard_4x4(8.0)
    sec = edlib.Sector(16, 8, 8, edlib.ED_HUBBARD, t=t, U=U)
    osec = O.Sector(16, 8, 8)
    rng = np.random.default_rng(7)
    x = rng.uniform(-0.5, 0.5, osec.dim)
    yref = O.hprod_hubbard_mt(osec, t, U, x)
    xd = sec.from_ref(torch.from_numpy(x).cuda())
    yd = torch.zeros_like(xd)
    sec.hv(xd, yd)
    y = sec.to_ref(yd).cpu().numpy()
    err = np.linalg.norm(y - yref) / np.linalg.norm(yref)
    assert err <= 1e-14, err
    del xd, yd, y, yref
    xi = O.hashvec(np.arange(osec.dim), 3, 1)
    yref = O.hprod_hubbard_mt(osec, t, U, xi)
    for dt in (torch.float64, torch.float32):
        xd = sec.from_ref(torch.from_numpy(xi).cuda().to(dt))
        yd = torch.zeros_like(xd)
        sec.hv(xd, yd)
        assert np.array_equal(sec.to_ref(yd).double().cpu().numpy(), yref), dt
        del xd, yd


def _heis_4x8(edlib):
    from pyhub_gb300.tools import lattices as LT
    J = LT.heisenberg_4x8(1.0)
    return J, edlib.Sector(32, 16, 0, edlib.ED_HEISENBERG, J=J)


def _sample_rows(dim, n=100_000, seed=11):
    rng = np.random.default_rng(seed)
    rows = rng.choice(dim, n, replace=False)
    return np.unique(np.concatenate([rows, [0, 1, dim // 2, dim - 2, dim - 1]]))


def test_heisenberg_4x8_sampled_rows_match_oracle(edlib):
    import torch
    J, sec = _heis_4x8(edlib)
    rows = _sample_rows(sec.dim)
    ridx = torch.from_numpy(rows).cuda()
    for kind in (0, 1):
        yref, ab = O.hprod_heis_rows(32, J, rows, 5, kind)
        for dt in ((torch.float64,) if kind == 0 else (torch.float64, torch.float32)):
            x = sec.from_ref(_hash_device(sec.dim, 5, kind, dt))
            y = torch.zeros_like(x)
            sec.hv(x, y)
            got = y[ridx].double().cpu().numpy()
            del x, y
            if kind == 0:
                assert np.all(np.abs(got - yref) <= 64 * EPS64 * ab), np.max(np.abs(got - yref) / ab)
            else:
                assert np.array_equal(got, yref), dt


def test_heisenberg_4x8_sampled_spin_correlations_match_oracle(edlib):
    import torch
    J, sec = _heis_4x8(edlib)
    rows = _sample_rows(sec.dim, seed=12)
    ridx = torch.from_numpy(rows).cuda()
    bonds = [(i + 1, j + 1) for i in range(32) for j in range(32) if i != j and J[i, j] != 0.0]
    pairs = bonds + [(1, 1), (17, 17), (32, 32)]
    for kind in (0, 1):
        ref, ab = O.j_spin_heis_rows(32, rows, 21, 22, kind, pairs)
        ket = sec.from_ref(_hash_device(sec.dim, 22, kind, torch.float64))
        full = sec.from_ref(_hash_device(sec.dim, 21, kind, torch.float64))
        bra = torch.zeros_like(full)
        bra[ridx] = full[ridx]
        del full
        raw, _ = sec.rdm_raw(bra, ket, pairs=pairs)
        got = raw[:, 0] + raw[:, 1]
        del bra, ket
        if kind == 0:
            assert np.all(np.abs(got - ref) <= 1e-12 * ab), np.max(np.abs(got - ref) / ab)
        else:
            assert np.array_equal(got, ref)


def _int_vector(sec, seed, dtype):
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    v = torch.randint(-3, 4, (sec.dim,), generator=g, device="cuda").to(torch.float64)
    return sec.from_ref(v).to(dtype)


def _check_exact_and_symmetric(edlib, sec):
    import torch
    x32 = _int_vector(sec, 1, torch.float32)
    y32 = torch.zeros_like(x32)
    sec.hv(x32, y32)
    x64 = x32.double()
    y64 = torch.zeros_like(x64)
    sec.hv(x64, y64)
    assert torch.equal(y32.double(), y64)
    del x32, y32
    x2 = _int_vector(sec, 2, torch.float64)
    y2 = torch.zeros_like(x2)
    sec.hv(x2, y2)
    a = float(torch.dot(x64, y2))
    b = float(torch.dot(y64, x2))
    assert abs(a - b) <= 1e-13 * max(abs(a), 1.0)


def test_hubbard_4x4_exact_and_symmetric(edlib):
    from pyhub_gb300.tools import lattices as LT
    t, U = LT.hubbard_4x4(8.0)
    sec = edlib.Sector(16, 8, 8, edlib.ED_HUBBARD, t=t, U=U)
    _check_exact_and_symmetric(edlib, sec)


def test_heisenberg_4x8_exact_and_symmetric(edlib):
    from pyhub_gb300.tools import lattices as LT
    sec = edlib.Sector(32, 16, 0, edlib.ED_HEISENBERG, J=LT.heisenberg_4x8(1.0))
    _check_exact_and_symmetric(edlib, sec)


def test_batched_lanczos_full_size_clusters(edlib):
    import torch
    from pyhub_gb300 import _capi
    from pyhub_gb300.core import greens_batched as GB
    from pyhub_gb300.core import lanczos as LZ
    cl = GB.c4_clusters(2, seed=0)
    secs, src = [], []
    for spec in cl:
        N = spec["N"]
        U = np.full(12, spec["U"])
        src.append(_capi.Sector(12, N, N, _capi.ED_HUBBARD, t=spec["t"], U=U))
        secs.append(_capi.Sector(12, N + 1, N, _capi.ED_HUBBARD, t=spec["t"], U=U))
        secs.append(_capi.Sector(12, N, N - 1, _capi.ED_HUBBARD, t=spec["t"], U=U))
    bl = GB.BatchedLanczos(secs, 30, dtype=torch.float64)
    kinds = ["e_up", "h_down"]
    for i, sec in enumerate(secs):
        c = i // 2
        psi = LZ.start_vector(src[c], seed=c, dtype=torch.float64)
        psi /= torch.linalg.vector_norm(psi)
        _capi.gf_start(src[c], sec, kinds[i % 2], 1 + i, psi, bl.start(i))
    starts = [bl.start(i).clone() for i in range(len(secs))]
    bl.run()
    torch.cuda.synchronize()
    A, B = bl.alpha.cpu().numpy(), bl.beta.cpu().numpy()
    for i, sec in enumerate(secs):
        a, b = GB.plain_coefficients(sec, starts[i], 30)
        n = np.count_nonzero(b[1:] > 1e-8)
        assert np.allclose(A[i, :n], a[:n], rtol=1e-9, atol=1e-9), i
        assert np.allclose(B[i, :n + 1], b[:n + 1], rtol=1e-9, atol=1e-9), i


def test_fp32_dots_and_norms_error_bound_at_4x4_length(edlib):
    """The FP32 multi-dot sums each warp's 512 products in FP32 (16 in sequence
    per thread, then 5 shuffle levels) before the FP64 stage, and the update's
    norm sums 16 squares per thread in FP32: deterministic bounds
    |dot - dot64| <= 22 u32 sum_i |v_i w_i| and |n2 - n2_64| <= 17 u32 n2_64
    (u32 = 2^-24), checked on 4x4-length vectors (165,636,900 elements)
    against FP64 torch sums of the same FP32 data."""
    import torch
    from pyhub_gb300 import _capi
    n = 12870 * 12870
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    nv = 3
    V = torch.rand((nv, n), generator=g, device="cuda", dtype=torch.float32) - 0.5
    V[2] += 0.25                       # a vector with a large mean: partial sums grow
    w = torch.rand(n, generator=g, device="cuda", dtype=torch.float32) - 0.5
    w += 0.1
    sc = torch.empty(_capi.scratch_bytes(n, nv) // 8 + 1, dtype=torch.float64, device="cuda")
    out = torch.zeros(nv, dtype=torch.float64, device="cuda")
    _capi.multidot(V, nv, w, out, sc)
    u32 = 2.0 ** -24
    for j in range(nv):
        vd, wd = V[j].double(), w.double()
        ref = float(torch.dot(vd, wd))
        absum = float(torch.dot(vd.abs(), wd.abs()))
        assert abs(float(out[j]) - ref) <= 22 * u32 * absum, (j, float(out[j]), ref)
    coef = torch.tensor([0.3, -0.2, 0.1], dtype=torch.float64, device="cuda")
    res = torch.empty(n, dtype=torch.float32, device="cuda")
    nrm = torch.zeros(1, dtype=torch.float64, device="cuda")
    _capi.update(V, nv, coef, w, res, norm2=nrm, scratch=sc)
    ref = float((res.double() ** 2).sum())
    assert abs(float(nrm[0]) - ref) <= 17 * u32 * ref
