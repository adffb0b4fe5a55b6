"""Save/restore of a Lanczos solve with reduced quantities and Green's
functions: the restored solver answers every property exactly as the one that
solved, without a new solve; the Ritz states come back bit for bit."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nup,ndn", [(4, 4), (4, 3)])
def test_lanczos_solve_save_restore(edlib, tmp_path, nup, ndn):
    import torch
    from pyhub_gb300.solver import FermiHubbard
    t = O.ring(8)
    fh = FermiHubbard(8, nup, ndn, t, 4.0)
    fh.kernel(max_lcz=200, acc_lcz=1e-8, compute_spgf=True, nb_sites_comp=3)
    assert fh.is_lanczos
    path = fh.save(str(tmp_path / "solver"))
    back = FermiHubbard(8, nup, ndn, t, 4.0).restore(path)
    assert back.is_lanczos and back.nb_lcz == fh.nb_lcz
    assert back.e0 == fh.e0
    np.testing.assert_array_equal(back.lcz_results["alpha"], fh.lcz_results["alpha"])
    np.testing.assert_array_equal(back.psi0, fh.psi0)
    assert torch.equal(back._state_device(0), fh._state_device(0))
    for spin in ("up", "down"):
        np.testing.assert_array_equal(back.one_rdm[spin], fh.one_rdm[spin])
    np.testing.assert_array_equal(back.spin_cor_matrix, fh.spin_cor_matrix)
    np.testing.assert_array_equal(back.nb_poles, fh.nb_poles)
    w = np.linspace(-6, 6, 65)
    g0, g1 = fh.gf_matrix(w, 0.1), back.gf_matrix(w, 0.1)
    for spin in ("up", "down"):
        assert torch.equal(g0[spin], g1[spin])
    # a quantity formed after the restore from the restored state: same kernel, same input
    raw0, _ = fh.sector(nup, ndn).rdm_raw(fh._state_device(0), pairs=[(1, 2)], flags=2)
    raw1, _ = back.sector(nup, ndn).rdm_raw(back._state_device(0), pairs=[(1, 2)], flags=2)
    np.testing.assert_array_equal(raw0, raw1)
