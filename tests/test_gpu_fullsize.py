"""Size-independent properties at the benchmark sizes, where the oracle is
too slow to compare against:

* 4x4 Hubbard (t=1, U=8, D=165,636,900) and 4x8 Heisenberg (J=1,
  D=601,080,390): with integer-valued inputs every partial sum is an exact
  FP32 number, so the FP32 and FP64 products must be equal bit for bit;
  and <x1, H x2> = <H x1, x2> (H symmetric) in FP64 to 1e-13 relative.
* two 12-site clusters of the batched Green's-function set: the batched
  alpha/beta equal the per-instance three-term Lanczos to 1e-9 (30 steps).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


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
