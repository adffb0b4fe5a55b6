"""The solver.h5 tree in an .npz archive: round trips of the store and of
CoreSolver.save/restore for a dense solve (host arrays only, no GPU)."""
import os

import numpy as np
import pytest

from pyhub_gb300.core import store
from pyhub_gb300.core.greens import PoleBlock
from pyhub_gb300.solver.fermi_hubbard import FermiHubbard


def test_store_round_trip(tmp_path):
    tree = {"@version": 2, "input": {"@nb_sites": 4, "@exec_name": "hubbard.x", "@flag": True, "@T": 0.25,
                                     "U": np.arange(4.0), "lanczos": {"@max_lcz": 600}},
            "solve": {"eigenvalues": np.linspace(-3, 1, 7), "empty": {}, "psi_0": np.ones(5, np.float32)}}
    path = store.save(str(tmp_path / "solver"), tree)
    assert path.endswith("solver.npz") and os.path.exists(path)
    back = store.load(path)
    assert back["@version"] == 2 and back["input"]["@exec_name"] == "hubbard.x"
    assert back["input"]["@flag"] and back["input"]["@T"] == 0.25
    assert back["input"]["lanczos"]["@max_lcz"] == 600
    np.testing.assert_array_equal(back["input"]["U"], np.arange(4.0))
    assert back["solve"]["empty"] == {}
    assert back["solve"]["psi_0"].dtype == np.float32
    # a second save replaces the archive and leaves no temporary file
    store.save(path, {"input": {"@nb_sites": 5}})
    assert store.load(path)["input"]["@nb_sites"] == 5
    assert sorted(os.listdir(tmp_path)) == ["solver.npz"]


@pytest.mark.parametrize("bad", [{"a/b": 1}, {"": 1}, {"@@x": 1}, {"@g": {"x": 1}}, {"o": np.array([{}], dtype=object)}])
def test_store_rejects_bad_trees(tmp_path, bad):
    with pytest.raises((ValueError, TypeError)):
        store.save(str(tmp_path / "x.npz"), bad)


def _dense_solver(U, nb=2):
    n = 4
    t = -np.eye(n, k=1) - np.eye(n, k=-1)
    t[0, -1] = t[-1, 0] = -1.0
    s = FermiHubbard(n, 2, 2, t, U=U, T=0.5)
    rng = np.random.default_rng(7)
    D = 36
    A = rng.normal(size=(D, D))
    val, vec = np.linalg.eigh(A + A.T)
    s.max_lcz, s.acc_lcz, s.nb_comp_states_, s.store_H, s.nb_sites_comp = 600, 1e-8, nb, True, n
    s._sol = {"eigenvalues": val, "eigenvectors_ref": vec, "is_lanczos": False, "deg": 1, "H": A + A.T, "nstates": D}
    s._sol["boltzmann"] = s._boltzmann(val, nb)
    s.is_solve = True
    s.set_state(-1)
    nw = len(s.wgt)
    s._rq = {"density_matrix_up": rng.normal(size=(nw, n, n)), "density_matrix_down": rng.normal(size=(nw, n, n)),
             "ni": rng.normal(size=(nw, n)), "sisj": rng.normal(size=(nw, n, n)),
             "dbl_occ": rng.normal(size=(nw, n, n, n, n)) if np.ndim(U) == 4 else None}
    s.is_reduced_quantities = True
    spgf = []
    for b in range(nw):
        blocks = {"up": {}}
        for part, sign in (("greater", 1.0), ("lesser", -1.0)):
            blk = PoleBlock(n, sign, float(val[b]))
            for i in range(n):
                m = 3 + i
                blk.diag[i] = (rng.normal(size=m), rng.uniform(size=m))
                blk.norm2[i] = float(rng.uniform())
            for i in range(n):
                for j in range(i + 1, n):
                    blk.pair[(i, j)] = (rng.normal(size=4), rng.uniform(size=4))
                    blk.norm2_pair[(i, j)] = float(rng.uniform())
            blocks["up"][part] = blk
        blocks["down"] = blocks["up"]
        spgf.append(blocks)
    s._spgf = spgf
    s.is_spgf = True
    s.gf = s.compute_gf()
    return s


def _uijkl(n=4):
    rng = np.random.default_rng(3)
    U = rng.normal(size=(n, n, n, n))
    return 0.5 * (U + np.einsum('ijkl->jilk', U))


@pytest.mark.parametrize("U", [4.0, "uijkl"])
def test_core_solver_save_restore_dense(tmp_path, U):
    U = _uijkl() if isinstance(U, str) else U
    a = _dense_solver(U)
    path = a.save(str(tmp_path / "solver"))
    b = FermiHubbard(4, 2, 2, a.t_matrix, U=U, T=0.5).restore(path)
    np.testing.assert_array_equal(b.e, a.e)
    assert b.e0 == a.e0 and b.nb_comp_states == a.nb_comp_states and b.nb_deg == a.nb_deg
    np.testing.assert_array_equal(b.H, a.H)
    np.testing.assert_array_equal(b._sol["eigenvectors_ref"], a._sol["eigenvectors_ref"])
    for spin in ("up", "down"):
        np.testing.assert_array_equal(b.one_rdm[spin], a.one_rdm[spin])
    np.testing.assert_array_equal(b.ni, a.ni)
    np.testing.assert_array_equal(b.spin_cor_matrix, a.spin_cor_matrix)
    if np.ndim(U) == 4:
        np.testing.assert_array_equal(b.two_rdm, a.two_rdm)
    assert b.e_two_body == a.e_two_body
    w = np.linspace(-4, 4, 33)
    for raw in (False, True):
        ga, gb = a.gf_matrix(w, 0.1, device="cpu", raw=raw), b.gf_matrix(w, 0.1, device="cpu", raw=raw)
        for spin in ("up", "down"):
            np.testing.assert_array_equal(gb[spin].numpy(), ga[spin].numpy())
    np.testing.assert_array_equal(b.nb_poles, a.nb_poles)


def test_archive_layout_is_the_references(tmp_path):
    """The reduced quantities are stored with the state index last, as the
    reference reads them (reduced_quantities.py:14-27, 48)."""
    U = _uijkl()
    a = _dense_solver(U)
    tree = store.load(a.save(str(tmp_path / "solver")))
    rq, w = tree["reduced_quantities"], a.wgt / np.sum(a.wgt)
    np.testing.assert_allclose(np.einsum('jki,i->jk', rq["density_matrix_up"], w), a.one_rdm["up"], rtol=1e-14)
    np.testing.assert_allclose(np.einsum('ji,i->j', rq["ni"], w), a.ni, rtol=1e-14)
    np.testing.assert_allclose(np.einsum('jki,i->jk', rq["sisj"], w), a.spin_cor_matrix, rtol=1e-14)
    np.testing.assert_allclose(np.einsum('ijklb,b->lkji', rq["dbl_occ"], w), a.two_rdm, rtol=1e-14)
    inp = tree["input"]
    assert inp["@is_Uloc"] == 3 and inp["@do_rq_two_body"]
    np.testing.assert_allclose(inp["Upartial"], np.einsum('ijkl,ijkl->ij', U, U))
    assert tree["solve"]["@nw"] == len(a.wgt) and tree["solve"]["@is_lanczos"] == 0
    np.testing.assert_array_equal(tree["solve"]["eigenvectors"][1], a._sol["eigenvectors_ref"][:, 1])


def test_restore_refuses_another_hamiltonian(tmp_path):
    a = _dense_solver(4.0)
    path = a.save(str(tmp_path / "solver"))
    with pytest.raises(ValueError, match="U differs"):
        FermiHubbard(4, 2, 2, a.t_matrix, U=5.0, T=0.5).restore(path)
    with pytest.raises(ValueError, match="T differs"):
        FermiHubbard(4, 2, 2, a.t_matrix, U=4.0, T=0.0).restore(path)
    with pytest.raises(ValueError, match="n_up differs"):
        FermiHubbard(4, 3, 2, a.t_matrix, U=4.0, T=0.5).restore(path)
    with pytest.raises(RuntimeError, match="kernel"):
        FermiHubbard(4, 2, 2, a.t_matrix, U=4.0).save(str(tmp_path / "none"))


def test_nvtx_range_without_a_device():
    from pyhub_gb300.trace import nvtx
    with nvtx("pyhub.test"):
        x = 1
    assert x == 1
    with pytest.raises(KeyError):
        with nvtx("pyhub.test"):
            raise KeyError("propagates")


def test_basis_file_helpers():
    from pyhub_gb300.core.basis import Basis
    b = Basis(4, hilbert=(2, 1))
    b.exec_basis([2, 1])
    assert b.file_size == 0.0
    b.__basisremove__()
    assert len(b.basis_up) == 6 and len(b.basis_down) == 4
