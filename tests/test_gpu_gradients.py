"""Gradients of E0 and of a 1-RDM loss with respect to every bond hopping,
on-site U and on-site energy: Hellmann-Feynman and the adjoint MINRES solve
against central finite differences (h = 1e-5) of the engine and of the FP64
oracle (dense diagonalisation).

Tolerances: dE0/dtheta 1e-6 absolute; dL/dtheta 2e-5 relative to max |dL/dtheta|.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _cluster(n, extra, seed):
    from pyhub_gb300.tools import lattices as LT
    return LT.random_bond_cluster(n, extra, seed)


def _oracle_e0_gamma(params, theta, nup, ndn):
    t, U = params.unpack(theta)
    sec = O.Sector(params.norb, nup, ndn)
    H = O.dense_h(lambda v: O.hprod_hubbard(sec, t, U, v, fast=True), sec.dim)
    e, v = np.linalg.eigh(H)
    g = O.one_rdm(sec, v[:, 0])
    return e[0], g, (sec, v[:, 0])


def test_hellmann_feynman_matches_oracle_fd(edlib):
    from pyhub_gb300.core import gradients as GR
    t, U, bonds = _cluster(6, 3, 7)
    P = GR.HubbardParams(6, bonds)
    theta = P.pack(t, U)
    sol = GR.solve(P, theta, 3, 3)
    g = GR.hf_gradient(P, sol)
    h = 1e-5
    for k in range(P.nparams):
        tp, tm = theta.copy(), theta.copy()
        tp[k] += h
        tm[k] -= h
        fd = (_oracle_e0_gamma(P, tp, 3, 3)[0] - _oracle_e0_gamma(P, tm, 3, 3)[0]) / (2 * h)
        assert abs(g[k] - fd) < 1e-6, (P.names()[k], g[k], fd)


def test_hellmann_feynman_matches_engine_fd_8_sites(edlib):
    from pyhub_gb300.core import gradients as GR
    t, U, bonds = _cluster(8, 4, 3)
    P = GR.HubbardParams(8, bonds)
    theta = P.pack(t, U)
    g = GR.hf_gradient(P, GR.solve(P, theta, 4, 4))
    h = 1e-5
    rng = np.random.default_rng(0)
    for k in rng.choice(P.nparams, size=8, replace=False):
        tp, tm = theta.copy(), theta.copy()
        tp[k] += h
        tm[k] -= h
        fd = (GR.solve(P, tp, 4, 4).e0 - GR.solve(P, tm, 4, 4).e0) / (2 * h)
        assert abs(g[k] - fd) < 1e-6, (P.names()[k], g[k], fd)


def test_rdm_loss_adjoint_matches_oracle_fd(edlib):
    from pyhub_gb300.core import gradients as GR
    t, U, bonds = _cluster(6, 3, 11)
    P = GR.HubbardParams(6, bonds)
    theta = P.pack(t, U)
    t2, U2, _ = _cluster(6, 3, 12)
    target = _oracle_e0_gamma(P, P.pack(t2, U2) * 0 + theta + 0.05, 3, 3)[1]
    sol = GR.solve(P, theta, 3, 3)
    L, g, info = GR.rdm_loss_gradient(P, sol, target)
    e0o, go, _ = _oracle_e0_gamma(P, theta, 3, 3)
    Lo = np.sum((go["up"] - target["up"]) ** 2) + np.sum((go["down"] - target["down"]) ** 2)
    assert abs(L - Lo) < 1e-10
    h = 1e-5

    def loss(th):
        gg = _oracle_e0_gamma(P, th, 3, 3)[1]
        return np.sum((gg["up"] - target["up"]) ** 2) + np.sum((gg["down"] - target["down"]) ** 2)

    fd = np.array([(loss(theta + h * e) - loss(theta - h * e)) / (2 * h) for e in np.eye(P.nparams)])
    assert np.abs(g - fd).max() < 2e-5 * max(1e-3, np.abs(fd).max()), (np.abs(g - fd).max(), np.abs(fd).max())
    assert info["minres_relres"] < 1e-9


def test_autograd_function(edlib):
    import torch
    from pyhub_gb300.core import gradients as GR
    t, U, bonds = _cluster(6, 2, 5)
    P = GR.HubbardParams(6, bonds)
    theta = torch.tensor(P.pack(t, U), requires_grad=True)
    E0 = GR.GroundStateEnergy.make(P, 3, 3)
    e = E0.apply(theta)
    e.backward()
    sol = GR.solve(P, theta.detach().numpy(), 3, 3)
    assert abs(float(e) - sol.e0) < 1e-10
    assert np.allclose(theta.grad.numpy(), GR.hf_gradient(P, sol), atol=1e-10)
