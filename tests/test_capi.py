"""CPU checks of the C-ABI library: it loads, exports every function that
include/pyhub_ed.h declares, and its host-only entry points (basis
enumeration, rank, argument validation) behave.  No kernel is launched."""
import ctypes
import os
import re

import numpy as np
import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(ed_[a-z0-9_]+)\s*\(", src))
    return names


def test_library_exports_every_declared_symbol(edlib):
    lib = ctypes.CDLL(os.path.join(ROOT, "pyhub_gb300", "libpyhub_ed.so"))
    declared = _declared()
    assert len(declared) >= 10
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing


@pytest.mark.parametrize("no,ne", [(8, 4), (12, 5), (16, 8), (20, 10), (5, 0), (5, 5), (32, 1)])
def test_basis_matches_oracle(edlib, no, ne):
    b = edlib.basis(no, ne)
    ref = O.hilbert(no, ne)
    assert np.array_equal(b, ref)
    for i in np.random.default_rng(0).choice(len(b), size=min(200, len(b)), replace=False):
        assert edlib.rank(no, ne, int(b[i])) == i


def test_binom_and_rank_edges(edlib):
    assert edlib.binom(32, 16) == 601080390
    assert edlib.rank(8, 4, 0b1111) == O.rank(8, 4, 0b1111)
    assert edlib.rank(8, 4, 0b111) == -1          # wrong particle number
    assert edlib.rank(8, 4, 0x1F0) == -1          # bits beyond norb


def test_invalid_arguments_rejected_before_launch(edlib):
    with pytest.raises(edlib.EDError) as e:
        edlib.Sector(40, 2, 2, edlib.ED_HUBBARD, t=np.zeros((40, 40)), U=np.zeros(40))
    assert e.value.code == edlib.ED_ERR_RANGE
    with pytest.raises(edlib.EDError):
        edlib.Sector(4, 2, 2, edlib.ED_HEISENBERG, J=np.zeros((4, 4)))  # sector must be (2, 0)
    t = np.zeros((4, 4))
    t[0, 1] = np.nan
    with pytest.raises(edlib.EDError, match="non-finite"):
        edlib.Sector(4, 2, 2, edlib.ED_HUBBARD, t=t, U=np.zeros(4))
    L = edlib.lib()
    assert L.ed_hv(None, None, 0, 0, None, None, 1.0, None, None, 0) == edlib.ED_ERR_ARG
    assert "NULL" in L.ed_last_error().decode()


def test_pointer_checks_refuse_host_and_short_tensors():
    """Tensors handed to kernels are checked on the host first: a CPU tensor,
    a strided last dimension or too few elements raise before any launch."""
    import torch
    from pyhub_gb300 import _capi
    with pytest.raises(ValueError, match="CUDA tensor"):
        _capi._ptr(torch.zeros(8), 4, "x")
    assert _capi._ptr(None) is None


def test_lanczos_state_size_and_limits(edlib):
    """ed_lanczos_state_doubles: stop code, Gram maximum, mmax+1 scales, the
    (mmax+1)^2 inverse Cholesky factor and four work vectors; -1 outside
    1..8192 (and the Python wrapper raises)."""
    L = edlib.lib()
    for m in (1, 200, 8192):
        assert L.ed_lanczos_state_doubles(m) == 3 + m + (m + 1) ** 2 + 4 * (m + 1)
    assert L.ed_lanczos_state_doubles(0) == -1 and L.ed_lanczos_state_doubles(8193) == -1
    with pytest.raises(ValueError):
        edlib.lanczos_state_doubles(9000)


def test_new_entry_points_reject_bad_arguments(edlib):
    """The device Lanczos step, the continued fractions, the multi-site start
    vectors and the kept-basis batch refuse bad arguments on the host, with a
    message, before any launch."""
    L = edlib.lib()
    ARG = edlib.ED_ERR_ARG
    assert L.ed_lanczos_coef(None, 0, 0, None, None, None, None, None, None) == ARG
    assert "mmax" in L.ed_last_error().decode()
    assert L.ed_lanczos_coef(None, 5, 4, None, None, None, None, None, None) == ARG   # k > mmax
    assert L.ed_cf_eval(None, 1, 0, None, None, 4, None, None, None, None) == ARG    # no levels
    assert L.ed_cf_eval(None, 1, 5000, None, None, 4, None, None, None, None) == ARG  # > 3000 levels
    assert "3000" in L.ed_last_error().decode()
    assert L.ed_cf_eval(None, 0, 10, None, None, 4, None, None, None, None) == edlib.ED_OK   # nothing to do
    sites = (ctypes.c_int32 * 40)(*range(1, 41))
    assert L.ed_gf_start_sites(None, None, None, 0, 40, sites, 0, 0, None, 0, 0, None, 0) == ARG
    assert "nsites" in L.ed_last_error().decode()
    assert L.ed_batch_ritz_sum(None, None, 0, None, 10, None, None, None) == ARG
    assert L.ed_batch_lanczos_kept(None, None, 0, None, None, None, 10, None, None, None, 0) == ARG


def test_composite_and_operator_entry_points_reject_bad_arguments(edlib):
    """The composite calls (one Lanczos step, the assembled RDMs, the
    Hellmann-Feynman gradient) and the operator engine refuse a missing
    sector, space or buffer, and a malformed operator space, with a message,
    before anything touches a GPU."""
    L = edlib.lib()
    ARG = edlib.ED_ERR_ARG
    assert L.ed_lanczos_step_scratch_bytes(None, 10) == 0
    assert L.ed_rdm1_scratch_bytes(None) == 0
    assert L.ed_lanczos_step(None, None, edlib.ED_F32, 0, None, 0, 0, 10, None, None, None, None, None, 0) == ARG
    assert "sector" in L.ed_last_error().decode()
    assert L.ed_rdm1(None, None, edlib.ED_F64, 0, None, None, None, None, None, 0) == ARG
    assert L.ed_hf_grad(None, None, edlib.ED_F64, 0, None, 0, None, None, None, None, None, 0) == ARG
    assert "Hubbard" in L.ed_last_error().decode()
    assert L.ed_ops_apply(None, None, 0, None, None, None, None, None, None, 0) == ARG
    assert "space" in L.ed_last_error().decode()
    out = ctypes.c_void_p()
    nu = (ctypes.c_int * 2)(2, 2)
    nd = (ctypes.c_int * 1)(1)
    assert L.ed_opspace_create(40, 1, nu, 1, nd, ctypes.byref(out)) == ARG        # more sites than 32
    assert "norb" in L.ed_last_error().decode()
    assert L.ed_opspace_create(4, 2, nu, 1, nd, ctypes.byref(out)) == ARG         # 2 listed twice
    assert "twice" in L.ed_last_error().decode()
    bad = (ctypes.c_int * 1)(5)
    assert L.ed_opspace_create(4, 1, bad, 1, nd, ctypes.byref(out)) == ARG        # 5 particles on 4 sites
    assert "outside" in L.ed_last_error().decode()
    assert not out.value
