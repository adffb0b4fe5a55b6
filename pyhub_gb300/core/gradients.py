"""Parameter gradients of the ground state on the GPU.

No reference counterpart: the reference offers no derivatives.  The
quantities involved are the reference's own (E0 of LANCZOS, the 1-RDM of
ONE_RDM, static_rq.f90:153-244), so the gradients are checked against
central finite differences of the engine and of the FP64 oracle.

Parameters theta of a Hubbard cluster with a fixed bond list:
  t_b  (b = (i,j), i<j)   symmetric hopping t_matrix[i,j] = t_matrix[j,i] = t_b
  U_i                     on-site interaction
  eps_i                   on-site energy, the diagonal of t_matrix (the reference
                          keeps it there, funcmod.f90:25 KINOP with J==K)
Hellmann-Feynman (one fused pass of the RDM kernel over psi):
  dE0/dt_b   = sum_s <c^+_is c_js + c^+_js c_is>
  dE0/deps_i = sum_s <n_is>
  dE0/dU_i   = <n_i,up n_i,down>
1-RDM loss L = sum_s ||gamma_s - gamma_s^target||_F^2 (gamma_s[i,j] = <c^+_is c_js>):
  dL/dpsi = 2 A psi with A = sum_s,ij G_ij c^+_is c_js, G = 2(gamma - target),
  applied as an H*v with t_matrix = G and U = 0;
  (H - E0) lambda = -P_perp dL/dpsi solved by MINRES on the orthogonal
  complement of psi (short recurrences: the Krylov basis is recomputed, never
  stored);
  dL/dtheta = <lambda| dH/dtheta |psi>, a transition RDM from the same kernel.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .. import _capi
from . import lanczos as LZ
from .reduced_quantities import all_pairs, lower_pairs, scatter_pairs


def _torch():
    import torch
    return torch


@dataclass
class HubbardParams:
    norb: int
    bonds: list          # [(i, j)] 0-based, i < j

    @property
    def nparams(self):
        return len(self.bonds) + 2 * self.norb

    def pack(self, t: np.ndarray, U: np.ndarray) -> np.ndarray:
        return np.concatenate([[t[i, j] for (i, j) in self.bonds], np.asarray(U, dtype=float), np.diag(t)])

    def unpack(self, theta):
        theta = np.asarray(theta, dtype=np.float64)
        nb = len(self.bonds)
        t = np.zeros((self.norb, self.norb))
        for k, (i, j) in enumerate(self.bonds):
            t[i, j] = t[j, i] = theta[k]
        U = theta[nb:nb + self.norb].copy()
        t[np.diag_indices(self.norb)] = theta[nb + self.norb:]
        return t, U

    def names(self):
        return ([f"t_{i}_{j}" for (i, j) in self.bonds] + [f"U_{i}" for i in range(self.norb)]
                + [f"eps_{i}" for i in range(self.norb)])

    def pairs(self):
        """Site pairs (1-based) whose RDM sums the gradient needs: both
        directions of every bond, then the diagonal."""
        pr = []
        for (i, j) in self.bonds:
            pr += [(i + 1, j + 1), (j + 1, i + 1)]
        pr += [(i + 1, i + 1) for i in range(self.norb)]
        return pr

    def contract(self, raw: np.ndarray) -> np.ndarray:
        """<bra| dH/dtheta |ket> for every parameter from the raw sums over pairs()."""
        nb = len(self.bonds)
        g = np.zeros(self.nparams)
        for k in range(nb):
            a, b = raw[2 * k], raw[2 * k + 1]
            g[k] = a[0] + b[0] + a[4] + b[4]           # up and down hops, both directions
        for i in range(self.norb):
            d = raw[2 * nb + i]
            g[nb + i] = d[3]                           # <n_up n_down>
            g[nb + self.norb + i] = d[0] + d[2]        # <n_up> + <n_down>
        return g


@dataclass
class Solution:
    e0: float
    psi: object          # FP64 device tensor, internal layout
    sector: object
    gamma: dict          # {'up': NxN, 'down': NxN}


def solve(params: HubbardParams, theta, nup: int, ndn: int, mode: str = "f64", steps: int = 400,
          seed: int = 0, tol: float = 1e-11) -> Solution:
    """Ground state (Lanczos until the Ritz residual |H psi - E0 psi| < tol) and
    the spin-resolved 1-RDM (computed, not copied, for both spins)."""
    t, U = params.unpack(theta)
    sec = _capi.Sector(params.norb, nup, ndn, _capi.ED_HUBBARD, t=t, U=U)
    # f64: one Lanczos run to the residual.  mixed: the FP32 stage stops near its own floor
    # (Ritz residual estimate 1e-5; the basis traffic grows with the square of the steps), and the
    # FP64 refinement runs to the residual tol (the 1-RDM and the adjoint need psi itself, which an
    # energy criterion converges only to its root)
    if mode == "f64":
        rule, refine = LZ.ResidualRule(tol, min_steps=10), None
    else:
        rule, refine = LZ.ResidualRule(max(tol, 1e-5), min_steps=20), LZ.ResidualRule(tol, min_steps=4)
    gs = LZ.ground_state(sec, mode=mode, steps=steps, seed=seed, rule=rule, refine_rule=refine)
    gamma = one_rdm(sec, gs.psi, params.norb)
    return Solution(e0=gs.e0, psi=gs.psi, sector=sec, gamma=gamma)


def one_rdm(sec, psi, norb: int, ket=None) -> dict:
    # <psi|c+_J c_K|psi> of a real state is symmetric: the pairs K <= J, mirrored (as ONE_RDM
    # forms it); a transition density <bra|.|ket> needs both orders and is symmetrised
    pairs = lower_pairs(norb) if ket is None else all_pairs(norb)
    raw, _ = sec.rdm_raw(psi, ket, pairs=pairs, flags=1)
    q = scatter_pairs(raw, pairs, norb).reshape(norb, norb, 6)
    # <c^+_J c_K> sums: q[J-1][K-1][0] for J != K (hop K -> J), diagonal <n_J>
    gu = q[:, :, 0].copy()
    gd = q[:, :, 4].copy()
    gd[np.diag_indices(norb)] = q[np.arange(norb), np.arange(norb), 2]
    if ket is None:
        low = np.tril_indices(norb, -1)
        gu.T[low] = gu[low]
        gd.T[low] = gd[low]
        return {"up": gu, "down": gd}
    return {"up": 0.5 * (gu + gu.T), "down": 0.5 * (gd + gd.T)}


def hf_gradient(params: HubbardParams, sol: Solution) -> np.ndarray:
    """dE0/dtheta by Hellmann-Feynman: one fused RDM pass over psi."""
    raw, _ = sol.sector.rdm_raw(sol.psi, pairs=params.pairs(), flags=1)
    return params.contract(raw)


def _apply_one_body(sol: Solution, G: np.ndarray, psi, out):
    """out = A psi, A = sum_{s,ij} G_ij c^+_is c_js (same G for both spins)."""
    norb = G.shape[0]
    Gs = 0.5 * (G + G.T)
    sec_a = _capi.Sector(norb, sol.sector.nup, sol.sector.ndn, _capi.ED_HUBBARD, t=Gs, U=np.zeros(norb))
    sec_a.hv(psi, out)
    return sec_a


def minres(apply, b, psi, maxiter: int = 2000, rtol: float = 1e-10):
    """MINRES (Paige and Saunders, SIAM J. Numer. Anal. 12, 1975) for the
    symmetric system (H - E0) x = b with b orthogonal to psi.  Every
    operator application is projected onto the complement of psi, the
    near-null direction of H - E0.  Three-term Lanczos recurrence with Givens
    rotations of its tridiagonal: work vectors only, no stored basis."""
    torch = _torch()

    def proj(v):
        v.sub_(psi * torch.dot(psi, v))
        return v

    x = torch.zeros_like(b)
    r = proj(b.clone())
    beta1 = float(torch.linalg.vector_norm(r).item())
    if beta1 == 0.0:
        return x, 0, 0.0
    v_prev = torch.zeros_like(b)
    v = r / beta1
    beta = 0.0
    dbar, epsln, cs, sn, phibar = 0.0, 0.0, -1.0, 0.0, beta1
    w = torch.zeros_like(b)
    w1 = torch.zeros_like(b)
    it = 0
    for it in range(1, maxiter + 1):
        p = proj(apply(v).clone())
        if beta != 0.0:
            p.sub_(beta * v_prev)
        alpha = float(torch.dot(v, p).item())
        p.sub_(alpha * v)
        beta_next = float(torch.linalg.vector_norm(p).item())
        oldeps = epsln
        delta = cs * dbar + sn * alpha
        gbar = sn * dbar - cs * alpha
        epsln = sn * beta_next
        dbar = -cs * beta_next
        gamma = math.hypot(gbar, beta_next)
        if gamma == 0.0:
            break
        cs, sn = gbar / gamma, beta_next / gamma
        phi = cs * phibar
        phibar = sn * phibar
        w_new = (v - oldeps * w1 - delta * w) / gamma
        w1, w = w, w_new
        x.add_(phi * w)
        if abs(phibar) <= rtol * beta1 or beta_next == 0.0:
            break
        v_prev, v = v, p / beta_next
        beta = beta_next
    return proj(x), it, abs(phibar) / beta1


def rdm_loss_gradient(params: HubbardParams, sol: Solution, target: dict, maxiter: int = 3000,
                      rtol: float = 1e-11):
    """L = sum_s ||gamma_s - target_s||^2 and dL/dtheta by the adjoint solve."""
    torch = _torch()
    gu, gd = sol.gamma["up"], sol.gamma["down"]
    L = float(np.sum((gu - target["up"]) ** 2) + np.sum((gd - target["down"]) ** 2))
    Gu, Gd = 2.0 * (gu - target["up"]), 2.0 * (gd - target["down"])
    # The one-body operator is applied through a sector product, which acts on both spins with one
    # matrix.  With N_up = N_down and spin-symmetric targets the two weights agree up to the solve's
    # rounding; their mean is applied, and a real asymmetry is refused.
    if np.abs(Gu - Gd).max() > 1e-4 * max(1.0, np.abs(Gu).max()):
        raise NotImplementedError("spin-dependent loss weights (gamma_up != gamma_down) are not supported")
    G = 0.5 * (Gu + Gd)
    psi = sol.psi
    Apsi = torch.zeros_like(psi)
    _apply_one_body(sol, G, psi, Apsi)
    b = -2.0 * Apsi
    work = torch.zeros_like(psi)

    def apply(v):
        sol.sector.hv(v, work)
        return work - sol.e0 * v

    lam, iters, relres = minres(apply, b, psi, maxiter=maxiter, rtol=rtol)
    # dH/dtheta is symmetric, so <lam|dH|psi> = <psi|dH|lam>: one transition pass
    raw, _ = sol.sector.rdm_raw(lam, psi, pairs=params.pairs(), flags=1)
    return L, params.contract(raw), {"minres_iters": iters, "minres_relres": relres}


class GroundStateEnergy:
    """torch.autograd.Function pair: E0(theta) with the Hellmann-Feynman backward,
    and L(theta) = sum_s ||gamma_s(theta) - target_s||^2 with the adjoint backward."""

    @staticmethod
    def make(params: HubbardParams, nup: int, ndn: int, mode: str = "f64", target: dict = None):
        torch = _torch()

        class _E0(torch.autograd.Function):
            @staticmethod
            def forward(ctx, theta):
                sol = solve(params, theta.detach().cpu().numpy(), nup, ndn, mode=mode)
                ctx.grad = torch.tensor(hf_gradient(params, sol), dtype=theta.dtype)
                return torch.tensor(sol.e0, dtype=theta.dtype)

            @staticmethod
            def backward(ctx, g):
                return g * ctx.grad

        class _Loss(torch.autograd.Function):
            @staticmethod
            def forward(ctx, theta):
                sol = solve(params, theta.detach().cpu().numpy(), nup, ndn, mode=mode)
                L, grad, _ = rdm_loss_gradient(params, sol, target)
                ctx.grad = torch.tensor(grad, dtype=theta.dtype)
                return torch.tensor(L, dtype=theta.dtype)

            @staticmethod
            def backward(ctx, g):
                return g * ctx.grad

        return _E0 if target is None else _Loss
