"""ed_multidot_noalloc: the multi-dot for callers that cannot allocate device
memory (and so cannot pass ed_multidot a scratch buffer) keeps its partial
sums in a fixed device array inside the library.  Called here through the
C ABI and checked against ed_multidot on two calls in a row (the second call
with different data, so a stale result from the shared array would show),
within the tolerance of the multi-dot tests: relative 1e-12.

This file is collected last on purpose: a failure here leaves every other
test already run."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bind(L):
    f = L.ed_multidot_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return f


@pytest.mark.parametrize("dt", ["f32", "f64"])
@pytest.mark.parametrize("with_z", [True, False])
@pytest.mark.parametrize("pad", [0, 32])
def test_multidot_noalloc_matches_multidot(edlib, dt, with_z, pad):
    """Both forms (dots with w and z, or w alone) and a padded vector stride."""
    import torch
    L = edlib.lib()
    f = _bind(L)
    td = torch.float32 if dt == "f32" else torch.float64
    code = edlib.ED_F32 if dt == "f32" else edlib.ED_F64
    n, nvec = 1_048_576 + 96, 9
    g = torch.Generator(device="cuda")
    g.manual_seed(7)
    V = torch.randn((nvec, n + pad), generator=g, dtype=td, device="cuda")   # row stride n + pad
    z = V[4, :n] if with_z else None
    m = 2 * nvec if with_z else nvec
    scratch = torch.empty(edlib.scratch_bytes(n, nvec) // 8 + 1, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        w = torch.randn(n, generator=g, dtype=td, device="cuda")
        ref = torch.zeros(m, dtype=torch.float64, device="cuda")
        edlib.multidot(V, nvec, w, ref, scratch, z=z, n=n)
        out = torch.full((m,), float("nan"), dtype=torch.float64, device="cuda")
        rc = f(stream, code, n, V.data_ptr(), V.stride(0), nvec, w.data_ptr(), None if z is None else z.data_ptr(),
               out.data_ptr())
        assert rc == edlib.ED_OK, L.ed_last_error().decode()
        torch.cuda.synchronize()
        r, o = ref.cpu().numpy(), out.cpu().numpy()
        assert np.all(np.isfinite(o))
        np.testing.assert_allclose(o, r, rtol=1e-12, atol=1e-12 * np.abs(r).max(), err_msg=f"call {call}")


def test_multidot_noalloc_empty_sizes_write_zeros(edlib):
    """n == 0 (or no vectors) launches nothing and leaves zeros in out."""
    import torch
    L = edlib.lib()
    f = _bind(L)
    V = torch.zeros((3, 64), dtype=torch.float32, device="cuda")
    out = torch.full((6,), float("nan"), dtype=torch.float64, device="cuda")
    rc = f(torch.cuda.current_stream().cuda_stream, edlib.ED_F32, 0, V.data_ptr(), 64, 3, V[0].data_ptr(),
           V[1].data_ptr(), out.data_ptr())
    assert rc == edlib.ED_OK, L.ed_last_error().decode()
    torch.cuda.synchronize()
    assert torch.count_nonzero(out) == 0


def test_multidot_noalloc_rejects_too_many_vectors(edlib):
    import torch
    L = edlib.lib()
    f = _bind(L)
    n, nvec = 4096, 65
    V = torch.zeros((nvec, n), dtype=torch.float32, device="cuda")
    w = torch.zeros(n, dtype=torch.float32, device="cuda")
    out = torch.zeros(nvec, dtype=torch.float64, device="cuda")
    rc = f(torch.cuda.current_stream().cuda_stream, edlib.ED_F32, n, V.data_ptr(), n, nvec, w.data_ptr(), None,
           out.data_ptr())
    assert rc == edlib.ED_ERR_RANGE
    assert "64" in L.ed_last_error().decode()
